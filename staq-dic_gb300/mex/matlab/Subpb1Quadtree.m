function [U, HPar, ALSub1Time, ConvItPerEle, LocalICGNBadPtNum] = Subpb1Quadtree(UOld, FOld, udual, vdual, ...
    coordinatesFEM, Df, ImgRef, ImgDef, mu, beta, HPar, ALSolveStep, DICpara, ICGNmethod, tol)
%SUBPB1QUADTREE The 2-DOF augmented-Lagrangian IC-GN step on the GPU (staqdic_mex).
%   The per-node loop and the bad-subset filter run in the library; U comes
%   back NaN at the bad subsets, which are filled within each 8-connected
%   region of DICpara.ImgRefMask.  HPar is passed through (the reference's
%   per-node solver recomputes it and does not return it).
if ~strcmp(ICGNmethod, 'GaussNewton')
    error('staqdic:args', 'Subpb1Quadtree: only ''GaussNewton'' is on the GPU path');
end
precision = 1;
if isfield(DICpara, 'staqdicPrecision'), precision = DICpara.staqdicPrecision; end
tic;
[U, ConvItPerEle, LocalICGNBadPtNum] = staqdic_mex('subpb1', double(UOld(:)), double(FOld(:)), ...
    double(udual(:)), double(vdual(:)), double(coordinatesFEM), Df.DfDx, Df.DfDy, Df.ImgRefMask, ImgRef, ...
    ImgDef, double(mu), double(beta), double(DICpara.winsize_List), double(tol), double(precision));
ALSub1Time = toc;
mask = Df.ImgRefMask;
if isfield(DICpara, 'ImgRefMask'), mask = DICpara.ImgRefMask; end
U = staqdic_fill_regions(U, [], coordinatesFEM, mask);
end

function [U, F, HtempPar, LocalTime, ConvItPerEle, LocalICGNBadPtNum, markCoordHoleStrain] = ...
    LocalICGNQuadtree(U0, coordinatesFEM, Df, ImgRef, ImgDef, DICpara, ICGNmethod, tol)
%LOCALICGNQUADTREE The local 6-DOF IC-GN pass on the GPU (staqdic_mex).
%   The per-node loop and the bad-subset filter run in the library (batched
%   FP32 form unless DICpara.staqdicPrecision = 0 asks for the plain FP64
%   drop-in); U and F come back NaN at the bad subsets, which are then filled
%   within each 8-connected region of the mask (staqdic_fill_regions).  Every
%   node takes DICpara.winsize, as in the reference; an optional
%   DICpara.winsize_per_node (N x 1) gives one subset size per node instead.
if ~strcmp(ICGNmethod, 'GaussNewton')
    error('staqdic:args', 'LocalICGNQuadtree: only ''GaussNewton'' is on the GPU path');
end
precision = 1;
if isfield(DICpara, 'staqdicPrecision'), precision = DICpara.staqdicPrecision; end
wl = [];
if isfield(DICpara, 'winsize_per_node'), wl = DICpara.winsize_per_node; end
ws = DICpara.winsize;
if numel(ws) > 1, ws = max(ws); end
tic;
[U, F, HtempPar, ConvItPerEle, markCoordHoleStrain, LocalICGNBadPtNum] = staqdic_mex('icgn_local', ...
    double(U0(:)), double(coordinatesFEM), Df.DfDx, Df.DfDy, Df.ImgRefMask, ImgRef, ImgDef, ...
    double(ws), double(wl), double(tol), double(precision));
LocalTime = toc;
[U, F] = staqdic_fill_regions(U, F, coordinatesFEM, Df.ImgRefMask);
end

function Uhat = Subpb2Quadtree(DICmesh, GaussPtOrder, beta, mu, U, F, udual, vdual, alpha, winstepsize, waitBarDisplayOrNot)
%SUBPB2QUADTREE The global FEM step on the GPU (staqdic_mex).
%   Hanging-node Q4 assembly and a Jacobi-preconditioned CG to a relative
%   residual of 1e-10 replace the direct solve.  The duals enter the
%   reference multiplied by zero, so they are not passed.
neumann = [];
if isfield(DICmesh, 'neumann'), neumann = DICmesh.neumann; end
dirichlet = [];
if isfield(DICmesh, 'dirichlet'), dirichlet = DICmesh.dirichlet; end
Uhat = staqdic_mex('subpb2', double(DICmesh.coordinatesFEM), double(DICmesh.elementsFEM), ...
    double(dirichlet(:)), double(neumann), double(GaussPtOrder), double(beta), double(mu), ...
    double(U(:)), double(F(:)), double(alpha), double(mean(winstepsize)));
end

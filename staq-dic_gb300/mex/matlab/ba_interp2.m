function Z = ba_interp2(F, X, Y, method)
%BA_INTERP2 Bicubic interpolation of F at (X, Y) on the GPU (staqdic_mex).
%   Same call and result as the reference's ba_interp2 MEX (ba_interp2.cpp):
%   Z has the shape of X followed by F's dimensions beyond the second; double
%   or single inputs, all of one class.  Only 'cubic' is implemented, as in
%   the reference's compiled source.
if nargin > 3 && ~strcmpi(method, 'cubic')
    error('staqdic:args', 'ba_interp2: only ''cubic'' is implemented');
end
Z = staqdic_mex('ba_interp2', F, X, Y);
end

function [x, y, u, v, cc] = funIntegerSearch(f, g, tempSizeOfSearchRegion, gridx, gridy, winsize, winstepsize, tempNoOfInitPt, varargin)
%FUNINTEGERSEARCH Whole-field integer search on the GPU (staqdic_mex).
%   The whole-field mode (tempNoOfInitPt = 0) of the reference: x, y, u, v and
%   cc.max are ny x nx (row = y); cc.qfactors is (nx*ny) x 2 in the point
%   order of the search (x fastest), cc.A is empty.  The seed-point mode
%   (tempNoOfInitPt = 1) is not on this path.
if tempNoOfInitPt ~= 0
    error('staqdic:args', 'funIntegerSearch: only the whole-field mode is on the GPU path');
end
S = tempSizeOfSearchRegion;
if numel(S) == 1, S = [S, S]; end
[x, y, u, v, ccmax, qf] = staqdic_mex('integer_search', double(f), double(g), double(S), ...
    double([gridx(1), gridx(end)]), double([gridy(1), gridy(end)]), double(winsize), double(winstepsize));
cc.max = ccmax;
cc.qfactors = qf;
cc.A = [];
end

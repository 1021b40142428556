function [xGrid, yGrid, uGrid, vGrid, cc] = funIntegerSearchMg(f, g, gridx, gridy, winsize, winstepsize, varargin)
%FUNINTEGERSEARCHMG Multigrid integer search on the GPU (staqdic_mex).
%   xGrid, yGrid, uGrid, vGrid and cc.max are ny x nx (row = y) on the node
%   grid the search chooses; cc.A is empty.  cc.qfactors (quality factors of
%   the last level's correlation maps) is not produced: IntegerSearch.m, the
%   caller on this path, does not read it.
[xGrid, yGrid, uGrid, vGrid, ccmax] = staqdic_mex('integer_search_mg', double(f), double(g), ...
    double([gridx(1), gridx(end)]), double([gridy(1), gridy(end)]), double(winsize(1)), double(winstepsize));
cc.max = ccmax;
cc.A = [];
end

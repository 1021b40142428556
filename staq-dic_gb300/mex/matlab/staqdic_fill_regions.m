function [U, F] = staqdic_fill_regions(U, F, coordinatesFEM, mask)
%STAQDIC_FILL_REGIONS Fill the NaN nodes of U (2N) and F (4N, may be empty).
%   The nodes are grouped by the 8-connected region of the mask that holds
%   their rounded position; within a region every component is interpolated
%   from the region's finite nodes (natural neighbour inside their hull,
%   nearest outside it), the way the local steps fill their bad subsets.
%   Nodes outside every region, or in a region with fewer than three finite
%   nodes, keep their values.
N = size(coordinatesFEM, 1);
px = round(coordinatesFEM(:, 1)); py = round(coordinatesFEM(:, 2));
inimg = px >= 1 & py >= 1 & px <= size(mask, 1) & py <= size(mask, 2);
lab = zeros(N, 1);
L = bwlabel(logical(mask), 8);
lab(inimg) = L(sub2ind(size(mask), px(inimg), py(inimg)));
nc = 2; comps = {U};
if ~isempty(F), nc = 6; comps = {U, F}; end
for r = 1:max(lab)
    nodes = find(lab == r);
    for k = 1:nc
        if k <= 2, vals = comps{1}; idx = 2 * nodes - 2 + k; else, vals = comps{2}; idx = 4 * nodes - 6 + k; end
        good = ~isnan(vals(idx));
        if all(good) || sum(good) < 3, continue; end
        it = scatteredInterpolant(coordinatesFEM(nodes(good), 1), coordinatesFEM(nodes(good), 2), ...
            vals(idx(good)), 'natural', 'nearest');
        vals(idx(~good)) = it(coordinatesFEM(nodes(~good), 1), coordinatesFEM(nodes(~good), 2));
        if k <= 2, comps{1} = vals; else, comps{2} = vals; end
    end
end
U = comps{1};
if ~isempty(F), F = comps{2}; end
end

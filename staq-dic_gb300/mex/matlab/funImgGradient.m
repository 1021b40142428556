function Df = funImgGradient(ImgRef, ImgDef, varargin)
%FUNIMGGRADIENT Image gradients of ImgRef on the GPU (staqdic_mex).
%   Df = funImgGradient(ImgRef, ImgDef, ImgRefMask) returns the fields of the
%   reference's finite-difference branch: DfCropWidth, DfAxis, imgSize,
%   ImgRefMask, and DfDx, DfDy (the 7-tap central differences on the image
%   cropped by 3 pixels, times the mask).  The 'splinecubic' branch is not on
%   this path.
imgSize = size(ImgRef);
if nargin > 2 && ~isempty(varargin{1})
    ImgRefMask = varargin{1};
else
    ImgRefMask = ones(imgSize(1), imgSize(2));
end
if nargin > 3 && strcmp(varargin{2}, 'splinecubic')
    error('staqdic:args', 'funImgGradient: the splinecubic branch is not on the GPU path');
end
Df.DfCropWidth = 3;
Df.DfAxis = [4, imgSize(1) - 3, 4, imgSize(2) - 3];
Df.imgSize = imgSize;
Df.ImgRefMask = ImgRefMask;
[Df.DfDx, Df.DfDy] = staqdic_mex('gradient', double(ImgRef), ImgRefMask);
end

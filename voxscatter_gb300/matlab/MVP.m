function JOut = MVP(JIn0, fN, Mr, Mc, Gram, transp_flag, idx, GPU_flag)
% JOut = MVP(JIn0, fN, Mr, Mc, Gram, transp_flag, idx, GPU_flag)
%
% The signature of src/src_vie/src_mvp/MVP.m:1 (= mv_AN_const.m), computed by
% libvoxscatter through voxscatter_mex:
%   JOut = Gram.*Mr.*JIn - Mc.*N(JIn)                   transp_flag 'notransp'
%   JOut = Gram.*conj(Mr).*JIn - conj(N(Mc.*conj(JIn))) transp_flag 'transp'
% on the unknowns idx (MATLAB's 1-based idx3).  The reference passes fN on
% every call; here the device operator made from fN, Mr, Mc and idx is kept
% between calls and rebuilt only when one of them changes, while Gram is
% passed with every call (it differs per incident direction and polarisation
% in the DDA drivers: 1/alpha_LDR).  GPU_flag is accepted and ignored: the GPU
% is always used.  JIn0 may hold several right-hand sides as columns.
persistent h key
k = vs_fingerprint(fN, Mr, Mc, idx);
if isempty(h) || ~isequal(k, key)
    if ~isempty(h)
        voxscatter_mex('op_destroy', h);
    end
    [L, M, N] = size(Mr);
    h = voxscatter_mex('op_create_fN', complex(fN), L, M, N, complex(Mr), complex(Mc), complex(1), double(idx(:)));
    key = k;
end
x = complex(reshape(JIn0, numel(idx), []));
nrhs = size(x, 2);
if isscalar(Gram)
    g = complex(repmat(Gram, nrhs, 1));
else
    g = complex(repmat(Gram(:), 1, nrhs));
end
JOut = voxscatter_mex('op_apply_gram', h, x, g, transp_flag, 'c128');
if nrhs == 1
    JOut = reshape(JOut, size(JIn0));
end
end

function k = vs_fingerprint(fN, Mr, Mc, idx)
% sizes and strided samples of the arguments that define the device operator
s = @(a) [numel(a), sum(abs(a(1:max(1, floor(numel(a) / 997)):end)))];
k = [size(fN), s(fN), s(Mr), s(Mc), s(double(idx))];
end

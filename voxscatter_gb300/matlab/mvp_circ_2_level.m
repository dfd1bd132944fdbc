function mvp = mvp_circ_2_level(inv_blocks, JIn, L, M, N, idx)
% mvp = mvp_circ_2_level(inv_blocks, JIn, L, M, N, idx)
%
% The signature of src/src_preconditioning/mvp_circ_2_level.m:2: the 2-level
% circulant preconditioner apply (FFT along x and y, one 3N x 3N block
% product per (x, y) frequency, inverse FFTs) on the unknowns idx, computed
% by libvoxscatter through voxscatter_mex.  inv_blocks is the reference's
% cell{L, M} of inverse blocks; the device preconditioner made from it is
% kept between calls and rebuilt only when the blocks or idx change.
persistent h key
k = [L, M, N, numel(idx), sum(abs(inv_blocks{1, 1}(:))), sum(abs(inv_blocks{L, M}(:))), sum(double(idx(:)))];
if isempty(h) || ~isequal(k, key)
    if ~isempty(h)
        voxscatter_mex('prec_destroy', h);
    end
    B = complex(zeros(3 * N, 3 * N, L, M));
    for i = 1:L
        for j = 1:M
            B(:, :, i, j) = inv_blocks{i, j};
        end
    end
    h = voxscatter_mex('prec_create_blocks', B, L, M, N, double(idx(:)));
    key = k;
end
mvp = reshape(voxscatter_mex('prec_apply', h, complex(JIn(:)), 'c128'), size(JIn));
end

function [x, flag, relres, iter, resvec] = vs_bicgstab(A, b, tol, maxit, M1, M2, x0)
% [x, flag, relres, iter, resvec] = vs_bicgstab(A, b, tol, maxit, M1, M2, x0)
%
% MATLAB's bicgstab(A, b, tol, maxit, M1, M2, x0) as the DDA drivers call it
% (main_DDA.m:82,120-121), with A a libvoxscatter operator handle and M1 a
% preconditioner handle or [] (applied on the right as MATLAB does): BiCGSTAB
% on the device, a c64 inner solve inside FP64 iterative refinement until
% the FP64 true residual is below tol.  Named vs_bicgstab so that MATLAB's
% own bicgstab stays callable.  iter counts half steps as 0.5; resvec holds
% the residual norms at every half step (absolute, as MATLAB's).
if nargin < 3 || isempty(tol), tol = 1e-6; end
if nargin < 4 || isempty(maxit), maxit = min(numel(b), 20); end
if nargin < 5, M1 = []; end
if nargin >= 6 && ~isempty(M2)
    error('voxscatter:bicgstab', 'a second preconditioner factor is not supported');
end
if nargin < 7, x0 = []; end
if isempty(M1), M1 = uint64([]); end
opts = struct('method', 'bicgstab', 'tol', tol, 'maxit', maxit);
[x, flag, relres, iter, resvec] = voxscatter_mex('solve', A, M1, complex(b(:)), complex(x0(:)), opts);
resvec = resvec * norm(b(:));
end

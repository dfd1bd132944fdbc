function [x, flag, relres, iter, resvec] = pgmresDR(A, b, restart, tol, maxit, ritz, L1, L2, R1, R2, x0)
% [x, flag, relres, iter, resvec] = pgmresDR(A, b, restart, tol, maxit, ritz, L1, L2, R1, R2, x0)
%
% The signature of src/src_numeric/src_iterative/pgmresDR.m:73, as the JVIE
% solvers call it (JVIE_Solver_const_GPU.m:400-447: one right preconditioner
% R1): GCRO-DR on the device, each cycle of `restart` Arnoldi steps recycling
% the `ritz` harmonic Ritz vectors of smallest magnitude; maxit counts the
% cycles after the first.  A is a libvoxscatter operator handle (from
% voxscatter_mex('op_create', ...)), R1 a preconditioner handle or [];
% L1, L2 and R2 must be empty.  iter = [steps of the last cycle, cycles
% after the first]; resvec holds the Arnoldi residual estimates relative to
% ||b||; relres is the true FP64 relative residual.
if ~isa(A, 'uint64')
    error('voxscatter:pgmresDR', 'A must be a libvoxscatter operator handle (voxscatter_mex(''op_create'', ...))');
end
if nargin < 6 || isempty(ritz), ritz = min(10, round(restart / 2)); end
if nargin < 7, L1 = []; end
if nargin < 8, L2 = []; end
if nargin < 9, R1 = []; end
if nargin < 10, R2 = []; end
if nargin < 11, x0 = []; end
if ~isempty(L1) || ~isempty(L2) || ~isempty(R2)
    error('voxscatter:pgmresDR', 'only the right preconditioner R1 is supported');
end
opts = struct('method', 'gmresdr', 'restart', restart, 'ritz', min(ritz, restart - 1), ...
              'tol', tol, 'maxit', restart * (maxit + 1));
if isempty(R1), R1 = uint64([]); end
[x, flag, relres, steps, resvec] = voxscatter_mex('solve', A, R1, complex(b(:)), complex(x0(:)), opts);
cycles = max(1, ceil(steps / restart));
iter = [steps - restart * (cycles - 1), cycles - 1];
end

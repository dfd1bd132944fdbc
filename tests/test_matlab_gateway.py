"""The MATLAB boundary as committed files: the MEX gateway compiles (syntax
and types, against a declaration stand-in of the documented MEX API, as
MATLAB is not installed here), dispatches every command it documents, calls
only entry points the C ABI header declares, and the .m shims keep the
reference's function signatures."""
import os
import re
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GW = os.path.join(ROOT, "voxscatter_gb300", "matlab", "voxscatter_mex.c")
MDIR = os.path.join(ROOT, "voxscatter_gb300", "matlab")


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
def test_gateway_compiles_against_the_documented_mex_api():
    r = subprocess.run(["gcc", "-std=c99", "-fsyntax-only", "-Wall", "-Wextra", "-Werror",
                        "-I", os.path.join(ROOT, "tests", "native"), "-I", os.path.join(ROOT, "include"), GW],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_gateway_dispatches_every_documented_command_and_uses_declared_entries():
    src = open(GW).read()
    documented = set(re.findall(r"voxscatter_mex\('([a-z_N]+)'", src))
    dispatched = set(re.findall(r'is\(cmd, "([a-z_N]+)"\)', src))
    assert documented and documented <= dispatched, documented - dispatched
    header = open(os.path.join(ROOT, "include", "voxscatter.h")).read()
    declared = set(re.findall(r"\b(vs_[a-z0-9_]+)\s*\(", header))
    called = set(re.findall(r"\b(vs_[a-z0-9_]+)\(", src))
    assert called <= declared, called - declared


# reference signatures (file:line in the reference) the shims keep
SIGNATURES = {
    "MVP.m": "function JOut = MVP(JIn0, fN, Mr, Mc, Gram, transp_flag, idx, GPU_flag)",  # src/src_vie/src_mvp/MVP.m:1
    "mvp_circ_2_level.m": "function mvp = mvp_circ_2_level(inv_blocks, JIn, L, M, N, idx)",  # mvp_circ_2_level.m:2
    "pgmresDR.m": "function [x, flag, relres, iter, resvec] = pgmresDR(A, b, restart, tol, maxit, ritz, L1, L2, "
                  "R1, R2, x0)",  # src/src_numeric/src_iterative/pgmresDR.m:73
    "vs_bicgstab.m": "function [x, flag, relres, iter, resvec] = vs_bicgstab(A, b, tol, maxit, M1, M2, x0)",
}


@pytest.mark.parametrize("name", sorted(SIGNATURES))
def test_shims_keep_the_reference_signatures(name):
    first = open(os.path.join(MDIR, name)).readline().strip()
    assert first == SIGNATURES[name]
    body = open(os.path.join(MDIR, name)).read()
    cmds = set(re.findall(r"voxscatter_mex\('([a-z_N]+)'", body))
    gw = set(re.findall(r'is\(cmd, "([a-z_N]+)"\)', open(GW).read()))
    assert cmds and cmds <= gw, cmds - gw

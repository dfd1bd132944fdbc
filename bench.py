#!/usr/bin/env python
"""Benchmark of the GB300 VoxScatter hot path.

One step = one complete solve of the hexagonal-plate DDA problem (diameter
8 lambda, thickness 2 lambda, m = 1.31+0.01i, grid 105x91x26, 558,714 unknowns)
to ||b - A x|| / ||b|| <= 1e-6 (true residual, FP64) with right-preconditioned
BiCGSTAB and the 2-level circulant preconditioner; mixed precision: the c64
matvec/preconditioner pipeline inside FP64 iterative refinement.  The same
solve with the c128 pipeline throughout is timed beside it.

  python bench.py [--gpus N --steps K --warmup W] [--impl reference]

Prints one JSON line (rank 0).  --impl reference times the FP64 NumPy/SciPy
restatement of the reference algorithm on the host cores.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "solve time to 1e-6 relative residual (BiCGSTAB + 2-level circulant preconditioner)"
TOL = 1e-6


def _max_over_ranks(value, dist, device):
    """The largest `value` over all ranks (a replicated job takes as long as
    its slowest rank); `value` itself without a process group."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def _workload():
    from voxscatter_gb300 import workloads as W
    p = W.config2()
    return p


def _config_dict(p, world=1):
    """The workload as both arms describe it (the FFT grid each arm embeds the
    same Toeplitz operator in is reported beside it as ``fft_grid``)."""
    L, M, N = p["L"], p["M"], p["N"]
    return {"workload": f"hex plate D=8 lambda, t=2 lambda, m=1.31+0.01i, grid {L}x{M}x{N}, "
                        f"{len(p['idx'])} dipoles, {3 * len(p['idx'])} unknowns, +z incidence, x-pol",
            "tol": TOL, "solver": "BiCGSTAB, right 2-level circulant preconditioner",
            "l2": "inputs larger than L2: preconditioner blocks (118.7 MB c64), Green spectrum and ~10 "
                  "solution-sized vectors, ~180 MB read per iteration against a 129 MB L2",
            "parallelism": f"replicas x{world}"}


def _peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            j = json.load(f)
        return float(j["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during a region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        if not self.lines:
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1])); mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def _pass_bytes(p, PQR, n3, e=8, sym=True, packed=False):
    """Algorithmic DRAM bytes of each launch of the c64 pipelines (one rhs);
    packed: the GEMV reads the padded lower triangles of the symmetric blocks."""
    L, M, N = p["L"], p["M"], p["N"]
    P, Q, R = PQR
    V = L * M * N
    i4 = 4
    G = 6 * (P // 2 + 1) * (Q // 2 + 1) * (R // 2 + 1) * e if sym else 6 * P * Q * R * e
    mv = [n3 * e + 3 * V * i4 + 3 * P * M * N * e,
          3 * P * M * N * e + 3 * P * Q * N * e,
          2 * 3 * P * Q * N * e + G,
          3 * P * Q * N * e + 3 * P * M * N * e,
          3 * P * M * N * e + 3 * V * i4 + 2 * n3 * e]
    n = 3 * N
    nblk = (L // 2 + 1) * (M // 2 + 1) if sym else L * M
    blk_elems = ((n * (n + 1) // 2 + 15) // 16 * 16) if packed else n * n
    pc = [n3 * e + 3 * V * i4 + 3 * V * e,
          2 * 3 * V * e,
          nblk * blk_elems * e + 2 * 3 * V * e,
          2 * 3 * V * e,
          3 * V * e + 3 * V * i4 + n3 * e]
    pinned = e * (9 * V + 1.5 * V + 12 * P * M * N + 12 * P * Q * N) + G
    return mv, pc, pinned


def _num_sms():
    import torch
    return torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count


def _apply_shapes(args, op, prec):
    if args.shapes:
        j = json.loads(args.shapes)
        if "op" in j:
            op.set_shape("c64", **j["op"])
        if "prec" in j:
            prec.set_shape("c64", **j["prec"])


def _pass_names(op, prec):
    """Kernel of each pipeline launch under the tuned c64 launch shapes."""
    so, sp = op.shape("c64"), prec.shape("c64")

    def xy(sh, pre):
        x2, y2 = sh["x_reg"] == 1, sh["y_reg"] == 1
        return (pre + ("k_x2_fwd" if x2 else "k_xf"), pre + ("k_s2_fwd" if y2 else "k_strided_fwd"),
                pre + ("k_s2_inv" if y2 else "k_strided_inv"), pre + ("k_x2_inv" if x2 else "k_xi"))
    a, b, c, d = xy(so, "")
    names_mv = [a, b, "k_z2" if so["z_reg"] in (1, 2) else "k_z", c, d]
    a, b, c, d = xy(sp, "prec_")
    if sp.get("fuse_xy") == 1:  # one plane kernel each way, passes 1 and 3 launch nothing
        a, b, c, d = "prec_k_plane_fwd", "none", "none", "prec_k_plane_inv"
    gemv = {1: "k_block_gemv_stream", 2: "k_block_gemv_packed"}.get(sp["gemv_mode"], "k_block_gemv_sym")
    names_pc = [a, b, gemv, c, d]
    return names_mv, names_pc


def _traffic_from_profiles(kernel):
    """DRAM bytes per launch of `kernel` from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "dram_traffic.txt")
    if not os.path.exists(path):
        return None
    for ln in open(path):
        f = ln.split()
        if len(f) >= 2 and f[0] == kernel:
            try:
                return float(f[1])
            except ValueError:
                return None
    return None


def _cpu_oracle_setup(p, workers):
    import oracle as O
    from oracle import _fft
    _fft.set_workers(workers)
    L, M, N = p["L"], p["M"], p["N"]
    nD = L * M * N
    idx = p["idx"]
    idx3 = np.concatenate([idx, nD + idx, 2 * nD + idx])
    Toep = O.green_toeplitz(p["r"], p["ko"])
    alpha = O.alpha_ldr(p["refInd"], p["ko"], p["d"], p["kvec"], p["Eo"])
    dV = p["d"] ** 3
    fN = O.fft_operator(O.circulant_nop_const(Toep))
    _, c1 = O.circ_1_level(Toep, L, M, N)
    _, blk = O.circ_2_level(c1, L, M, N)
    inv = O.invert_blocks(blk, 1 / alpha, dV)
    del blk
    chi = np.zeros(nD); chi[idx] = 1
    chi = chi.reshape((L, M, N), order="F")
    ones = np.ones((L, M, N))
    b = O.PlaneWavePointWise(p["Eo"], p["kvec"], p["r"]).ravel(order="F")[idx3]
    A = lambda v: O.MVP(v, fN, ones, dV * chi, 1 / alpha, "notransp", idx3)
    Pm = lambda v: O.mvp_circ_2_level(inv, v, L, M, N, idx3)
    return A, Pm, b


def _cpu_iteration_seconds(A, Pm, b, iters):
    import oracle as O
    t0 = time.perf_counter()
    _, flag, relres, it, _ = O.bicgstab(A, b, 1e-30, iters, Pm)
    return (time.perf_counter() - t0) / max(it, 1)


def run_reference(args):
    rank = _env_int("RANK", 0)
    if rank != 0:
        return 0
    p = _workload()
    workers = os.cpu_count() or 1
    A, Pm, b = _cpu_oracle_setup(p, workers)
    import oracle as O
    # iterations the FP64 reference algorithm needs (one untimed full solve)
    x, flag, relres, it_needed, _ = O.bicgstab(A, b, TOL, 2000, Pm)
    sample_iters = 2
    for _ in range(args.warmup):
        _cpu_iteration_seconds(A, Pm, b, sample_iters)
    per = [_cpu_iteration_seconds(A, Pm, b, sample_iters) for _ in range(args.steps)]
    per_it = float(np.median(per))
    value_ms = per_it * it_needed * 1e3
    sample = (f"one replica's solve on rank 0: {sample_iters} BiCGSTAB iterations per step of the FP64 "
              f"NumPy/SciPy restatement "
              f"(scipy.fft workers={workers}); solve = median s/iteration x {it_needed} iterations "
              f"(full untimed reference solve: flag {flag}, relres {relres:.2e})")
    line = {"impl": "reference", "metric": METRIC, "value": value_ms, "unit": "ms", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": per_it * sample_iters * 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "c128",
            "data": "synthetic (seeded reference-rule geometry)", "config": _config_dict(p, args.gpus),
            "fft_grid": "x".join(str(2 * v) for v in (p["L"], p["M"], p["N"])),
            "iterations": it_needed,
            "cpu_baseline": {"value": value_ms, "unit": "ms", "cores": workers, "kind": "port", "sample": sample},
            "e2e": {"value": value_ms, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


def _directions(seed, count):
    """`count` seeded incident directions, two polarisations each."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        v = rng.normal(size=3); v /= np.linalg.norm(v)
        a = np.cross(v, [0, 0, 1.0] if abs(v[2]) < 0.9 else [1.0, 0, 0]); a /= np.linalg.norm(a)
        out.append((v, a)); out.append((v, np.cross(v, a)))
    return out


def _krylov_variants(api, stream, op, prec, b_dev, x_dev, steps):
    """Mixed solves of the same plate with the reference's other Krylov
    drivers: GMRES(20) (main_DDA.m:128-129) and GCRO-DR(20, 5 recycled
    vectors) (pgmresDR.m, right preconditioned as the JVIE solvers call it)."""
    import torch
    out = {}
    for name, kw in (("gmres20", dict(method="gmres", restart=20)),
                     ("gmres_dr20_5", dict(method="gmres_dr", restart=20, ritz=5))):
        with torch.cuda.stream(stream):
            x_dev.zero_()
        api.solve_device(op, b_dev.data_ptr(), x_dev.data_ptr(), prec, tol=TOL, precision="mixed", **kw)
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(steps):
            with torch.cuda.stream(stream):
                x_dev.zero_()
            info = api.solve_device(op, b_dev.data_ptr(), x_dev.data_ptr(), prec, tol=TOL, precision="mixed", **kw)
        ev1.record(stream)
        ev1.synchronize()
        out[name] = {"ms": ev0.elapsed_time(ev1) / steps, "iterations": info["iter"], "relres": info["relres"],
                     "converged": info["flag"] == 0, "refinements": info["refinements"]}
    return out


def _batched(api, ctx, stream, p, op, prec, steps):
    """16 right-hand sides (8 directions x 2 polarisations) of the plate, one
    batched mixed solve; and the 32-plate x 16-rhs configuration (512 rhs)."""
    import torch
    from voxscatter_gb300 import workloads as W
    out = {}
    pairs = _directions(7, 8)
    B = np.array([api.plane_wave(op, p["r"], p["ko"] * v, pol) for v, pol in pairs])
    # each direction and polarisation has its own alpha_LDR (getOPERATOR_DDA.m:14-26)
    gram = np.array([1 / api.alpha_ldr(p["refInd"], p["ko"], p["d"], p["ko"] * v, pol) for v, pol in pairs])
    Bd = torch.from_numpy(B).cuda()
    Xd = torch.zeros_like(Bd)
    torch.cuda.synchronize()
    api.solve_batch_device(op, Bd.data_ptr(), Xd.data_ptr(), len(B), prec, tol=TOL, gram=gram)  # warm-up / capture
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(steps):
        with torch.cuda.stream(stream):
            Xd.zero_()
        infos = api.solve_batch_device(op, Bd.data_ptr(), Xd.data_ptr(), len(B), prec, tol=TOL, gram=gram)
    ev1.record(stream)
    ev1.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    out["plate_16rhs"] = {"ms_per_batch": ms, "ms_per_rhs": ms / len(B),
                          "converged": all(i["flag"] == 0 for i in infos),
                          "max_relres": max(i["relres"] for i in infos),
                          "max_iterations": max(i["iter"] for i in infos)}
    # 32 plates, diameters U[1,6] lambda (seeded), 16 rhs each (8 directions x
    # 2 polarisations, each with its own alpha_LDR), all on one context
    t0 = time.perf_counter()
    parts = []
    for q in W.config3_particles(seed=0):
        L, M, N = q["L"], q["M"], q["N"]
        nD = L * M * N
        idx3 = np.concatenate([q["idx"], nD + q["idx"], 2 * nD + q["idx"]])
        dV = q["d"] ** 3
        Tq = api.green_dda(q["r"], q["ko"], ctx=ctx)
        ainv = 1 / api.alpha_ldr(q["refInd"], q["ko"], q["d"], q["kvec"], q["Eo"])
        opq = api.Operator(L, M, N, idx3, 1.0, dV, ainv, toep=Tq, ctx=ctx)
        # the preconditioner is built for the +z, x-polarised alpha; each rhs solves its own system
        prq = api.Preconditioner(opq, shift=ainv, d=dV, precisions=("c64", "c128"))
        Bq = np.array([api.plane_wave(opq, q["r"], q["ko"] * v, pol) for v, pol in q["rhs"]])
        gq = np.array([1 / api.alpha_ldr(q["refInd"], q["ko"], q["d"], q["ko"] * v, pol) for v, pol in q["rhs"]])
        parts.append(dict(op=opq, pr=prq, B=torch.from_numpy(Bq).cuda(), nr=len(Bq), nv=len(q["idx"]), gram=gq))
    torch.cuda.synchronize()
    setup = (time.perf_counter() - t0) * 1e3
    Xs = [torch.zeros_like(q["B"]) for q in parts]
    for q, Xq in zip(parts, Xs):  # warm-up (graph capture per operator)
        api.solve_batch_device(q["op"], q["B"].data_ptr(), Xq.data_ptr(), q["nr"], q["pr"], tol=TOL, gram=q["gram"])
    torch.cuda.synchronize()

    def zero_all():
        for Xq in Xs:
            Xq.zero_()
        torch.cuda.synchronize()

    # one particle after another (each call returns with the stream idle)
    ev0.record(stream)
    conv, worst, iters = True, 0.0, []
    for _ in range(steps):
        zero_all()
        iters = []
        for q, Xq in zip(parts, Xs):
            inf = api.solve_batch_device(q["op"], q["B"].data_ptr(), Xq.data_ptr(), q["nr"], q["pr"], tol=TOL,
                                         gram=q["gram"])
            conv = conv and all(i["flag"] == 0 for i in inf)
            worst = max(worst, max(i["relres"] for i in inf))
            iters += [i["iter"] for i in inf]
    ev1.record(stream)
    ev1.synchronize()
    ms_seq = ev0.elapsed_time(ev1) / steps
    # all 32 plates in lockstep: one graph launch per inner iteration of all of them
    args_p = ([q["op"] for q in parts], [q["pr"] for q in parts], [q["B"].data_ptr() for q in parts],
              [Xq.data_ptr() for Xq in Xs], [q["nr"] for q in parts])
    grams = [q["gram"] for q in parts]
    zero_all()
    api.solve_particles(*args_p, grams=grams, tol=TOL)  # warm-up / capture
    torch.cuda.synchronize()
    ev0.record(stream)
    cconv, cworst = True, 0.0
    for _ in range(steps):
        zero_all()
        for inf in api.solve_particles(*args_p, grams=grams, tol=TOL):
            cconv = cconv and all(i["flag"] == 0 for i in inf)
            cworst = max(cworst, max(i["relres"] for i in inf))
    ev1.record(stream)
    ev1.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    nrhs = sum(q["nr"] for q in parts)
    out["plates32_512rhs"] = {"ms_total": ms, "ms_per_rhs": ms / nrhs, "rhs": nrhs, "particles": len(parts),
                              "solver": "vs_solve_particles (lockstep, one graph per inner iteration)",
                              "dipoles": int(sum(q["nv"] for q in parts)), "setup_ms": setup, "converged": cconv,
                              "max_relres": cworst, "sequential_ms_total": ms_seq, "sequential_converged": conv,
                              "sequential_max_relres": worst, "speedup_vs_sequential": ms_seq / ms,
                              "iterations_mean": float(np.mean(iters)), "iterations_max": float(np.max(iters))}
    return out


def run_ours(args):
    import torch
    rank = _env_int("RANK", 0)
    world = _env_int("WORLD_SIZE", 1)
    local = _env_int("LOCAL_RANK", 0)
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from voxscatter_gb300 import api
    ctx = api.Context(local)
    stream = torch.cuda.ExternalStream(ctx.stream_ptr())

    p = _workload()
    L, M, N = p["L"], p["M"], p["N"]
    nD = L * M * N
    idx = p["idx"]
    idx3 = np.concatenate([idx, nD + idx, 2 * nD + idx])
    dV = p["d"] ** 3
    t0 = time.perf_counter()
    Toep = api.green_dda(p["r"], p["ko"], ctx=ctx)
    alpha = api.alpha_ldr(p["refInd"], p["ko"], p["d"], p["kvec"], p["Eo"])
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep, ctx=ctx)
    prec = api.Preconditioner(op, shift=1 / alpha, d=dV, precisions=("c64", "c128"))
    ctx.synchronize()
    setup_ms = (time.perf_counter() - t0) * 1e3
    _apply_shapes(args, op, prec)
    n3 = op.n3
    bh = np.exp(1j * (p["kvec"][0] * p["r"][..., 0] + p["kvec"][1] * p["r"][..., 1] + p["kvec"][2] * p["r"][..., 2]))
    b_host = np.zeros(3 * nD, dtype=np.complex128)
    for c in range(3):
        b_host[c * nD:(c + 1) * nD] = p["Eo"][c] * bh.ravel(order="F")
    b_host = b_host[idx3]
    b_dev = torch.from_numpy(b_host).cuda()
    x_dev = torch.zeros_like(b_dev)
    torch.cuda.synchronize()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
        ctx.synchronize()

    def timed(precision, steps):
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        infos = []
        barrier()
        ev0.record(stream)
        for _ in range(steps):
            with torch.cuda.stream(stream):
                x_dev.zero_()
            infos.append(api.solve_device(op, b_dev.data_ptr(), x_dev.data_ptr(), prec, tol=TOL,
                                          precision=precision))
        ev1.record(stream)
        ev1.synchronize()
        ms = _max_over_ranks(ev0.elapsed_time(ev1) / steps, dist, "cuda")
        return ms, infos

    for _ in range(args.warmup):
        with torch.cuda.stream(stream):
            x_dev.zero_()
        api.solve_device(op, b_dev.data_ptr(), x_dev.data_ptr(), prec, tol=TOL, precision="mixed")
    with ClockSampler(local) as clk:
        ms_mixed, infos = timed("mixed", args.steps)
    launches = int(np.mean([i["launches"] for i in infos]))
    last = infos[-1]
    ok = all(i["flag"] == 0 and i["relres"] <= TOL for i in infos)

    # plain FP64 GPU path (same kernels in c128), fewer steps
    api.solve_device(op, b_dev.data_ptr(), x_dev.data_ptr(), prec, tol=TOL, precision="fp64")
    ms_fp64, infos64 = timed("fp64", max(1, min(args.steps, 3)))
    x_fp64 = x_dev.cpu().numpy()

    # end to end through the host-buffer C API with pinned host memory
    b_pin = torch.from_numpy(b_host).pin_memory()
    x_pin = torch.zeros_like(b_pin).pin_memory()
    e2e = []
    for k in range(args.warmup + args.steps):
        x_pin.zero_()
        barrier()
        t1 = time.perf_counter()
        api.solve_host_ptr(op, b_pin.data_ptr(), x_pin.data_ptr(), prec, tol=TOL, precision="mixed")
        if k >= args.warmup:
            e2e.append((time.perf_counter() - t1) * 1e3)
    e2e_ms = float(np.mean(e2e))

    # one more (untimed) mixed solve inside an NVTX range, so a profiler can be
    # limited to exactly one solve's launches (ncu --nvtx --nvtx-include "solve/")
    with torch.cuda.stream(stream):
        x_dev.zero_()
    ctx.synchronize()
    torch.cuda.nvtx.range_push("solve")
    api.solve_device(op, b_dev.data_ptr(), x_dev.data_ptr(), prec, tol=TOL, precision="mixed")
    ctx.synchronize()
    torch.cuda.nvtx.range_pop()
    x_mixed = x_dev.cpu().numpy()

    # one more mixed solve with CUDA events between the launches of its
    # captured iterations: every pass's duration inside the solve itself
    # (vs_solve_opts.profile_ms; the event nodes add a little, so it is not timed)
    with torch.cuda.stream(stream):
        x_dev.zero_()
    ctx.synchronize()
    prof = api.solve_device(op, b_dev.data_ptr(), x_dev.data_ptr(), prec, tol=TOL, precision="mixed",
                            profile=True)["profile"]

    # per-launch timing of the pipeline passes (c64), each pass alone
    xs = torch.randn(n3, dtype=torch.complex64, device="cuda")
    ys = torch.empty_like(xs)
    torch.cuda.synchronize()
    mv_ms = op.time_passes(xs.data_ptr(), ys.data_ptr(), 1, "c64", 50)
    pc_ms = prec.time_passes(xs.data_ptr(), ys.data_ptr(), 1, "c64", 50)
    mv_bytes, pc_bytes, pinned = _pass_bytes(p, op.PQR, n3, packed=prec.shape("c64")["gemv_mode"] == 2)
    names_mv, names_pc = _pass_names(op, prec)
    keys = api.PROFILE_KEYS
    in_solve = [prof[k] for k in keys]
    # the dominant HBM-bound launch and its roofline: CUDA events around one
    # launch of each pass on the library's stream (mean of 50), its duration
    # inside the solve's graph beside it
    allk = [(names_pc[i], pc_ms[i], pc_bytes[i], in_solve[i]) for i in range(5)] + \
           [(names_mv[i], mv_ms[i], mv_bytes[i], in_solve[5 + i]) for i in range(5)]
    dom = max(allk, key=lambda t: t[1])
    peak, peak_kind = _peaks()
    achieved = dom[2] / (dom[1] * 1e-3) / 1e9
    roof = {"bound": "hbm", "kernel": dom[0], "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_kind,
            "bytes_per_launch": dom[2], "ms_per_launch": dom[1],
            "ms_source": "CUDA events around one launch on the library's stream, mean of 50",
            "ms_per_launch_in_solve": dom[3],
            "traffic": _traffic_from_profiles(dom[0])}
    if dom[0].startswith("k_block_gemv_stream"):
        # the forward y pass before the GEMV prefetches the block every GEMV CTA
        # starts on into L2, so those bytes reach this launch from L2: the
        # HBM-served share of the algorithmic bytes over the same time beside it
        sh = prec.shape("c64")
        n = 3 * p["N"]
        nblk = (p["L"] // 2 + 1) * (p["M"] // 2 + 1)
        ctas = min(sh.get("gemv_blocks") or 2, 4)
        pf = min(nblk, _num_sms() * ctas) * n * n * 8 // 16 * 16 if sh.get("gemv_mode") == 1 else 0
        roof["l2_prefetched_bytes"] = pf
        roof["frac_hbm_served"] = (dom[2] - pf) / (dom[1] * 1e-3) / 1e9 / peak
    per_iter = 2 * sum(in_solve) + prof["solver_kernels_per_iter"]
    in_solve_line = {
        "source": "CUDA event nodes between the launches of one solve's captured iterations "
                  "(vs_solve_opts.profile_ms); each interval also holds one event node, so the "
                  "absolutes run a few us high and the shares are the figures to read",
        "per_iteration_ms": per_iter, "iterations_profiled": prof["iterations"],
        "passes_ms": dict(zip(keys, in_solve)), "solver_kernels_per_iter_ms": prof["solver_kernels_per_iter"],
        "share_of_iteration": {**{k: 2 * v / per_iter for k, v in zip(keys, in_solve)},
                               "solver_kernels": prof["solver_kernels_per_iter"] / per_iter},
        "fp64_residual_ms": prof["fp64_residual"], "fp64_residual_calls": prof["fp64_residual_calls"]}
    mv_total = sum(mv_ms)
    # the same pipeline on a batch of 16 right-hand sides (8 directions x 2
    # polarisations share one operator): intermediates 16x, spectrum read once
    nb16 = 16
    xb = torch.randn(nb16 * n3, dtype=torch.complex64, device="cuda")
    yb = torch.empty_like(xb)
    torch.cuda.synchronize()
    mv16 = op.time_passes(xb.data_ptr(), yb.data_ptr(), nb16, "c64", 20)
    per_rhs = 8 * (9 * nD + 1.5 * nD + 12 * op.PQR[0] * M * N + 12 * op.PQR[0] * op.PQR[1] * N)
    b16 = pinned + (nb16 - 1) * per_rhs
    del xb, yb
    # compulsory bytes: read x and write y once, the three diagonals, the spectrum once
    compulsory = 8 * 7.5 * nD + (pinned - per_rhs)
    matvec = {"ms": mv_total, "pinned_model_bytes": pinned, "GBps_pinned_model": pinned / (mv_total * 1e-3) / 1e9,
              "compulsory_bytes": compulsory, "GBps_compulsory": compulsory / (mv_total * 1e-3) / 1e9,
              "GBps_own_passes": sum(mv_bytes) / (mv_total * 1e-3) / 1e9, "passes_ms": mv_ms,
              "prec_apply_ms": sum(pc_ms), "prec_passes_ms": pc_ms,
              "prec_GBps": sum(pc_bytes) / (sum(pc_ms) * 1e-3) / 1e9,
              "batched16": {"ms": sum(mv16), "ms_per_rhs": sum(mv16) / nb16, "passes_ms": mv16,
                            "pinned_model_bytes": b16, "GBps_pinned_model": b16 / (sum(mv16) * 1e-3) / 1e9,
                            "frac_of_measured_hbm": b16 / (sum(mv16) * 1e-3) / 1e9 / peak}}

    batched = _batched(api, ctx, stream, p, op, prec, max(1, min(args.steps, 2))) if not args.no_batched else None
    koch = _koch_summary(api, ctx, max(2, min(args.steps, 5)), maxit=100) if not args.no_koch else None
    variants = _krylov_variants(api, stream, op, prec, b_dev, x_dev, max(1, min(args.steps, 2)))

    line = {"metric": METRIC, "value": ms_mixed, "unit": "ms", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_mixed, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None,
            "dtype": "c64 (inner products: exact float products summed in float-float; refinement residual on "
                     "FP64 data, its FFTs in double-float where faster; FP64 norms)",
            "data": "synthetic (seeded reference-rule geometry, plane-wave RHS)",
            "config": _config_dict(p, world), "fft_grid": "x".join(str(v) for v in op.PQR),
            "converged": ok, "relres": last["relres"], "iterations": last["iter"],
            "refinements": last["refinements"],
            "fp64_solve_ms": ms_fp64, "fp64_iterations": infos64[-1]["iter"],
            "speedup_mixed_vs_fp64": ms_fp64 / ms_mixed, "setup_ms": setup_ms,
            "roofline": roof, "in_solve": in_solve_line, "matvec": matvec,
            "shapes": {"op": op.shape("c64"), "prec": prec.shape("c64")},
            "e2e": {"value": e2e_ms, "unit": "ms", "h2d_bytes_per_step": int(b_pin.numel() * 16 * 2),
                    "d2h_bytes_per_step": int(x_pin.numel() * 16)},
            "gpu_launches": launches * args.steps, "clocks": clk.summary(), "batched": batched,
            "koch_256x256x64": koch,
            "krylov_variants": variants}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # one full FP64 solve of the same plate by the NumPy/SciPy restatement on
        # the host cores: the CPU baseline, and the FP64 reference solution that
        # the GPU solutions' field and C_ext errors are stated against
        import oracle as O
        workers = os.cpu_count() or 1
        A, Pm, b = _cpu_oracle_setup(p, workers)
        t1 = time.perf_counter()
        xo, fo, ro, ito, _ = O.bicgstab(A, b, TOL, 2000, Pm)
        cpu_ms = (time.perf_counter() - t1) * 1e3
        line["cpu_baseline"] = {
            "value": cpu_ms, "unit": "ms", "cores": workers, "kind": "port",
            "sample": f"one full BiCGSTAB solve to {TOL:g} of the FP64 NumPy/SciPy restatement "
                      f"(scipy.fft workers={workers}): {ito} iterations, flag {fo}, relres {ro:.2e}"}
        dV = p["d"] ** 3
        c_o = O.cext_dda(xo, b, p["ko"], dV, p["Eo"])
        acc = {"oracle_iterations": ito, "oracle_relres": ro, "cext_oracle": c_o}
        for name, xs in (("mixed", x_mixed), ("fp64", x_fp64)):
            c_g = api.cext(op, xs, b, p["ko"], dV, p["Eo"])
            acc[name] = {"field_rel_err": float(np.linalg.norm(xs - xo) / np.linalg.norm(xo)),
                         "cext": c_g, "cext_rel_err": abs(c_g - c_o) / abs(c_o),
                         "true_relres_fp64_oracle": float(np.linalg.norm(b - A(xs)) / np.linalg.norm(b))}
        line["accuracy_vs_fp64_oracle"] = acc
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_passes(args):
    """Setup + per-pass timing only (c64 and c128 matvec, c64 preconditioner)."""
    import torch
    from voxscatter_gb300 import api
    ctx = api.Context(0)
    p = _workload()
    L, M, N = p["L"], p["M"], p["N"]
    nD = L * M * N
    idx = p["idx"]
    idx3 = np.concatenate([idx, nD + idx, 2 * nD + idx])
    dV = p["d"] ** 3
    Toep = api.green_dda(p["r"], p["ko"], ctx=ctx)
    alpha = api.alpha_ldr(p["refInd"], p["ko"], p["d"], p["kvec"], p["Eo"])
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep, ctx=ctx)
    prec = api.Preconditioner(op, shift=1 / alpha, d=dV, precisions=("c64",))
    _apply_shapes(args, op, prec)
    xs = torch.randn(op.n3, dtype=torch.complex64, device="cuda")
    ys = torch.empty_like(xs)
    torch.cuda.synchronize()
    # each pipeline launch once more inside an NVTX range (ncu --nvtx --nvtx-include "passes/")
    op.time_passes(xs.data_ptr(), ys.data_ptr(), 1, "c64", 1)
    prec.time_passes(xs.data_ptr(), ys.data_ptr(), 1, "c64", 1)
    ctx.synchronize()
    torch.cuda.nvtx.range_push("passes")
    op.time_passes(xs.data_ptr(), ys.data_ptr(), 1, "c64", 1)
    prec.time_passes(xs.data_ptr(), ys.data_ptr(), 1, "c64", 1)
    ctx.synchronize()
    torch.cuda.nvtx.range_pop()
    names_mv, names_pc = _pass_names(op, prec)
    xd = torch.randn(op.n3, dtype=torch.complex128, device="cuda")
    yd = torch.empty_like(xd)
    torch.cuda.synchronize()
    out = {"fft_grid": op.PQR, "op_shape": op.shape("c64"), "prec_shape": prec.shape("c64"),
           "op_shape_c128": op.shape("c128"),
           "matvec_c128_ms": op.time_passes(xd.data_ptr(), yd.data_ptr(), 1, "c128", max(3, args.steps // 4)),
           "kernels": names_mv + names_pc,
           "matvec_c64_ms": op.time_passes(xs.data_ptr(), ys.data_ptr(), 1, "c64", args.steps),
           "prec_c64_ms": prec.time_passes(xs.data_ptr(), ys.data_ptr(), 1, "c64", args.steps)}
    if args.sweep:
        tuned_op, tuned_pr = op.shape("c64"), prec.shape("c64")
        zs = {}
        for z_reg in (0, 1, 2):
            for lg in ((2, 3, 4, 5) if z_reg == 0 else (4,)):
                op.set_shape("c64", z_reg=z_reg, lg_tile_z=lg)
                zs[f"z_reg={z_reg},lg_tile_z={lg}"] = op.time_passes(xs.data_ptr(), ys.data_ptr(), 1, "c64",
                                                                     args.steps)[2]
        op.set_shape("c64", **tuned_op)
        gs = {}
        for b in (1, 2, 4):
            for th in (64, 128, 256):
                prec.set_shape("c64", gemv_mode=0, gemv_blocks=b, gemv_threads=th, gemv_chunk=0)
                gs[f"direct,blocks={b},threads={th}"] = prec.time_passes(xs.data_ptr(), ys.data_ptr(), 1, "c64",
                                                                         args.steps)[2]
        n = 3 * N
        for b in (1, 2, 3, 4):
            for cq in (0, 8, 16, 32, (n + 1) // 2):
                prec.set_shape("c64", gemv_mode=1, gemv_blocks=b, gemv_threads=0, gemv_chunk=cq)
                gs[f"stream,ctas={b},chunk={cq}"] = prec.time_passes(xs.data_ptr(), ys.data_ptr(), 1, "c64",
                                                                     args.steps)[2]
        try:  # packed symmetric blocks, where the preconditioner has them
            for b in (1, 2, 3, 4):
                for ns in (2, 3, 4, 6, 8):
                    prec.set_shape("c64", gemv_mode=2, gemv_blocks=b, gemv_threads=0, gemv_chunk=ns)
                    gs[f"packed,ctas={b},stages={ns}"] = prec.time_passes(xs.data_ptr(), ys.data_ptr(), 1, "c64",
                                                                          args.steps)[2]
        except Exception as e:  # noqa: BLE001 - reported, not fatal
            gs["packed"] = f"unavailable: {e}"
        prec.set_shape("c64", **tuned_pr)
        ys_ = {}
        for yr in (0, 1):
            op.set_shape("c64", y_reg=yr)
            t = op.time_passes(xs.data_ptr(), ys.data_ptr(), 1, "c64", args.steps)
            prec.set_shape("c64", y_reg=yr)
            tp = prec.time_passes(xs.data_ptr(), ys.data_ptr(), 1, "c64", args.steps)
            ys_[f"y_reg={yr}"] = {"matvec": [t[1], t[3]], "prec": [tp[1], tp[3]]}
        op.set_shape("c64", **tuned_op)
        prec.set_shape("c64", **tuned_pr)
        out["y_pass_ms"] = ys_
        out["z_pass_ms"] = zs
        out["gemv_ms"] = gs
    print(json.dumps(out), flush=True)
    return 0


def run_adjoint(args):
    """64x64x16 random-permittivity slab (eps = (1.5+0.02i)^2 (1 + 0.1 g), g a
    seeded Gaussian random field of correlation length 4 voxels), z incidence,
    x polarisation: forward + plain-transpose adjoint solves for C_ext and
    dC_ext/deps per voxel, mixed and FP64; the FP64 gradient checked by central
    differences (h = 1e-6, re and im) on 16 seeded voxels.  One JSON line."""
    import torch
    from voxscatter_gb300 import api, workloads as W
    ctx = api.Context(0)
    p = W.config4(seed=0)
    L, M, N = p["L"], p["M"], p["N"]
    nD = L * M * N
    idx = p["idx"]
    idx3 = np.concatenate([idx, nD + idx, 2 * nD + idx])
    d, ko = p["d"], p["ko"]
    t = time.perf_counter()
    Toep = api.green_dda(p["r"], ko, ctx=ctx)
    ainv = 1 / api.alpha_ldr(p["eps"], ko, d, p["kvec"], p["Eo"], is_eps=True)
    G = np.zeros(nD, complex); G[idx] = ainv
    op = api.Operator(L, M, N, idx3, 1.0, d ** 3, G.reshape((L, M, N), order="F"), toep=Toep, ctx=ctx)
    pr = api.Preconditioner(op, shift=np.mean(ainv), d=d ** 3, precisions=("c64", "c128"))
    ctx.synchronize()
    setup_s = time.perf_counter() - t
    b = api.plane_wave(op, p["r"], p["kvec"], p["Eo"])
    res = {}
    for prec_name, tol in (("mixed", 1e-6), ("fp64", 1e-12)):
        api.cext_grad(op, pr, b, p["eps"], ko, d, p["kvec"], p["Eo"], tol=tol, precision=prec_name)  # warm-up
        times = []
        for _ in range(max(1, args.steps)):
            ctx.synchronize()
            t = time.perf_counter()
            c, gre, gim, P, i1, i2 = api.cext_grad(op, pr, b, p["eps"], ko, d, p["kvec"], p["Eo"], tol=tol,
                                                   precision=prec_name)
            times.append((time.perf_counter() - t) * 1e3)
        res[prec_name] = dict(c=c, gre=gre, gim=gim, P=P, ms=float(np.median(times)), it=(i1["iter"], i2["iter"]),
                              flags=(i1["flag"], i2["flag"]))
    f = res["fp64"]
    sc = max(np.abs(f["gre"]).max(), np.abs(f["gim"]).max())

    def cext_of(eps):
        ai = 1 / api.alpha_ldr(eps, ko, d, p["kvec"], p["Eo"], is_eps=True)
        G2 = np.zeros(nD, complex); G2[idx] = ai
        o2 = api.Operator(L, M, N, idx3, 1.0, d ** 3, G2.reshape((L, M, N), order="F"), toep=Toep, ctx=ctx)
        x, info, _ = api.solve(o2, b, pr, tol=1e-12, precision="fp64", x0=f["P"], want_resvec=False)
        return api.cext(o2, x, b, ko, d ** 3, p["Eo"])

    h = 1e-6
    rng = np.random.default_rng(1234)
    worst = 0.0
    t = time.perf_counter()
    for j in rng.choice(len(idx), 16, replace=False):
        for step, g in ((h, f["gre"]), (1j * h, f["gim"])):
            ep = p["eps"].copy(); ep[j] += step
            em = p["eps"].copy(); em[j] -= step
            worst = max(worst, abs((cext_of(ep) - cext_of(em)) / (2 * h) - g[j]) / sc)
    fd_s = time.perf_counter() - t
    m = res["mixed"]
    line = {"metric": "adjoint C_ext gradient: forward + adjoint solve time", "unit": "ms",
            "config": {"workload": f"random-permittivity slab {L}x{M}x{N}, {len(idx)} dipoles, eps=(1.5+0.02i)^2"
                                   f"(1+0.1 g), correlation length 4 voxels, seeded; z incidence, x polarisation"},
            "setup_s": setup_s, "cext": f["c"],
            "mixed": {"ms": m["ms"], "iterations_fwd_adj": m["it"], "flags": m["flags"],
                      "cext_rel_err_vs_fp64": abs(m["c"] - f["c"]) / abs(f["c"]),
                      "grad_max_err_vs_fp64": float(max(np.abs(m["gre"] - f["gre"]).max(),
                                                        np.abs(m["gim"] - f["gim"]).max()) / sc)},
            "fp64": {"ms": f["ms"], "iterations_fwd_adj": f["it"], "flags": f["flags"]},
            "central_differences": {"h": h, "voxels": 16, "worst_abs_err_over_max_grad": worst, "seconds": fd_s},
            "data": "synthetic (seeded random permittivity field)"}
    print(json.dumps(line), flush=True)
    return 0


def _koch_summary(api, ctx, steps, maxit=200, with_lu=True):
    """256x256x64 Koch snowflake (level 3, 16 central layers, m = 1.78+0.005i):
    setup times (Green tensor, operator, c64 preconditioner -- its 16,641
    blocks of 192 inverted on the tensor cores by default), the block inversion
    on the tensor cores against the CUDA cores, per-launch pipeline times, the
    matvec's model bandwidth and a bounded mixed GMRES(50) solve (this system
    converges slowly: relres after the iteration budget is reported)."""
    import torch
    from voxscatter_gb300 import workloads as W
    p = W.config5()
    L, M, N = p["L"], p["M"], p["N"]
    nD = L * M * N
    idx = p["idx"]
    idx3 = np.concatenate([idx, nD + idx, 2 * nD + idx])
    dV = p["d"] ** 3
    t = time.perf_counter()
    Toep = api.green_dda(p["r"], p["ko"], ctx=ctx)
    ctx.synchronize()
    green_s = time.perf_counter() - t
    alpha = api.alpha_ldr(p["refInd"], p["ko"], p["d"], p["kvec"], p["Eo"])
    t = time.perf_counter()
    op = api.Operator(L, M, N, idx3, 1.0, dV, 1 / alpha, toep=Toep, ctx=ctx)
    ctx.synchronize()
    op_s = time.perf_counter() - t
    t = time.perf_counter()
    prec = api.Preconditioner(op, shift=1 / alpha, d=dV, precisions=("c64",))
    ctx.synchronize()
    prec_s = time.perf_counter() - t
    n3 = op.n3
    xs = torch.randn(n3, dtype=torch.complex64, device="cuda")
    ys = torch.empty_like(xs)
    torch.cuda.synchronize()
    mv = op.time_passes(xs.data_ptr(), ys.data_ptr(), 1, "c64", steps)
    pc = prec.time_passes(xs.data_ptr(), ys.data_ptr(), 1, "c64", steps)
    mv_bytes, pc_bytes, pinned = _pass_bytes(p, op.PQR, n3)
    b = api.plane_wave(op, p["r"], p["kvec"], p["Eo"])
    bd = torch.from_numpy(np.ascontiguousarray(b)).cuda()
    xd = torch.zeros_like(bd)
    api.solve_device(op, bd.data_ptr(), xd.data_ptr(), prec, tol=1e-6, maxit=50, precision="mixed",
                     method="gmres", restart=50)
    xd.zero_()
    ctx.synchronize()
    t = time.perf_counter()
    info = api.solve_device(op, bd.data_ptr(), xd.data_ptr(), prec, tol=1e-6, maxit=maxit, precision="mixed",
                            method="gmres", restart=50)
    ctx.synchronize()
    solve_ms = (time.perf_counter() - t) * 1e3
    peak, peak_kind = _peaks()
    mv_ms = sum(mv)
    out = {"workload": f"Koch snowflake level 3, grid {L}x{M}x{N}, {len(idx)} dipoles, {n3} unknowns, "
                       f"m=1.78+0.005i", "fft_grid": "x".join(map(str, op.PQR)),
           "setup_s": {"green": green_s, "operator": op_s, "preconditioner_c64": prec_s},
           "shapes": {"op": op.shape("c64"), "prec": prec.shape("c64")},
           "matvec_c64_ms": mv, "prec_c64_ms": pc,
           "matvec_model_bytes": pinned, "matvec_model_GBps": pinned / (mv_ms * 1e-3) / 1e9,
           "matvec_model_frac": pinned / (mv_ms * 1e-3) / 1e9 / peak, "peak_GBps": peak, "peak_source": peak_kind,
           "gemv_GBps": pc_bytes[2] / (pc[2] * 1e-3) / 1e9,
           "gmres50": {"maxit": maxit, "ms": solve_ms, "ms_per_iteration": solve_ms / max(1.0, info["iter"]),
                       "flag": info["flag"], "relres": info["relres"], "iter": info["iter"]}}
    del op, prec, xs, ys, bd, xd
    if with_lu:
        out["block_inversion"] = _lu_cases(api, ctx, steps, 2, cases=(("snowflake_192", 192, 16641),))
    return out


def _lu_cases(api, ctx, steps, warmup, cases=(("snowflake_192", 192, 16641), ("hexplate_78", 78, 2523)),
              batch_cap=0):
    """The batched block inversion on the tensor cores against the CUDA-core
    blocked kernel, CUDA events on the context's stream, seeded
    well-conditioned FP32 blocks of the configurations' sizes."""
    import torch
    ext = torch.cuda.ExternalStream(ctx.stream_ptr())
    out = {}
    for name, n, nmat in cases:
        if batch_cap:
            nmat = min(nmat, batch_cap)
        g = torch.Generator(device="cuda").manual_seed(0)
        A = (torch.randn(nmat, n, n, dtype=torch.complex64, device="cuda", generator=g) * (0.5 / n ** 0.5)
             + torch.eye(n, dtype=torch.complex64, device="cuda") * (1.0 + 0.3j))
        Wk = torch.empty_like(A)
        res = {"n": n, "blocks": nmat, "flops_per_block": 8 * n ** 3}
        for method in ("tc", "cuda"):
            for _ in range(warmup):
                Wk.copy_(A)
                torch.cuda.synchronize()
                api.invert_blocks_device(Wk.data_ptr(), n, nmat, method, ctx=ctx)
            times = []
            for _ in range(steps):
                Wk.copy_(A)
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(ext)
                api.invert_blocks_device(Wk.data_ptr(), n, nmat, method, ctx=ctx)
                e1.record(ext)
                e1.synchronize()
                times.append(e0.elapsed_time(e1))
            ms = float(np.median(times))
            idx = np.linspace(0, nmat - 1, 8).astype(int)
            Ah = A[idx].cpu().numpy().astype(np.complex128)
            Wh = Wk[idx].cpu().numpy().astype(np.complex128)
            err = max(np.linalg.norm(Wh[k] - np.linalg.inv(Ah[k])) / np.linalg.norm(np.linalg.inv(Ah[k]))
                      for k in range(len(idx)))
            res[method] = {"ms": ms, "TFLOPs": 8 * n ** 3 * nmat / (ms * 1e-3) / 1e12, "max_rel_err_vs_fp64": err}
        res["speedup_tc_vs_cuda"] = res["cuda"]["ms"] / res["tc"]["ms"]
        out[name] = res
        del A, Wk
    return out


def run_koch(args):
    """256x256x64 Koch snowflake: one JSON line (see _koch_summary)."""
    from voxscatter_gb300 import api
    ctx = api.Context(0)
    line = {"metric": "koch 256x256x64: setup, pipeline launch times and bounded GMRES(50)", "unit": "ms"}
    line.update(_koch_summary(api, ctx, args.steps))
    print(json.dumps(line), flush=True)
    return 0

def run_lu(args):
    """Batched inversion of the preconditioner blocks (the parfor of inv() at
    main_DDA.m:107-111 / main_koch.m:114-118) on the tensor cores against the
    CUDA-core blocked Gauss-Jordan: the 256x256x64 snowflake's 16,641 stored
    blocks of 192 and the 105x91x26 plate's 2,523 blocks of 78, FP32 complex,
    seeded well-conditioned matrices of those sizes in HBM (values do not
    change the work).  --lu-batch limits the batch (small cases for profiling).
    One JSON line."""
    from voxscatter_gb300 import api
    ctx = api.Context(0)
    out = _lu_cases(api, ctx, args.steps, args.warmup, batch_cap=args.lu_batch)
    print(json.dumps({"metric": "batched block inversion (preconditioner build), FP32 complex", "unit": "ms",
                      "steps": args.steps, "warmup": args.warmup, "results": out}), flush=True)
    return 0

def run_nop(args):
    """Galerkin N-operator Toeplitz assembly (far + medium cells of
    assembly_nop_const.m) on a 128x128x64 grid: device time, against the FP64
    NumPy restatement timed on a sample of offsets (scaled to the grid)."""
    from voxscatter_gb300 import api
    from oracle import nop
    ctx = api.Context(0)
    L, M, N, ko, dx = 128, 128, 64, 2 * np.pi, 0.05
    api.nop_assemble(8, 8, 8, ko, dx, ctx=ctx)
    ts = []
    for _ in range(max(1, args.steps)):
        t = time.perf_counter()
        api.nop_assemble(L, M, N, ko, dx, ctx=ctx)
        ts.append(time.perf_counter() - t)
    Rf = nop.cube_faces(dx)
    W, U, V = nop.gauss_2d(nop.NP_FAR)
    rng = np.random.default_rng(0)
    offs = rng.integers(5, [L, M, N], size=(200, 3))
    t = time.perf_counter()
    for o in offs:
        nop.cubature_nop(W, U, V, o * dx, np.zeros(3), Rf, ko, dx)
    cpu_per_offset = (time.perf_counter() - t) / len(offs)
    line = {"metric": "N-operator Toeplitz assembly (far + medium face-pair cubature), 128x128x64", "unit": "s",
            "value": float(np.median(ts)), "offsets": L * M * N,
            "point_pairs": L * M * N * 21 * 256, "cpu_baseline": {
                "value": cpu_per_offset * L * M * N, "unit": "s", "cores": 1, "kind": "port",
                "sample": "200 far-cell offsets of the NumPy restatement (4x4 rule), scaled to 1,048,576 offsets"}}
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched (16- and 512-rhs) measurements")
    ap.add_argument("--no-koch", action="store_true", help="skip the 256x256x64 snowflake section of the main line")
    ap.add_argument("--sweep", action="store_true", help="passes mode: also time every z-pass and GEMV shape")
    ap.add_argument("--shapes", default=None,
                    help='JSON {"op": {...}, "prec": {...}} c64 launch shapes applied after autotuning '
                         '(replays a tuned configuration, e.g. under a profiler)')
    ap.add_argument("--lu-batch", type=int, default=0, help="lu mode: at most this many blocks per case")
    ap.add_argument("--mode", default="solve", choices=["solve", "passes", "koch", "nop", "adjoint", "lu"],
                    help="passes: only build the operator/preconditioner and time each pipeline launch "
                         "(a short command for ncu captures); koch: the 256x256x64 snowflake's pipeline "
                         "times and a bounded GMRES(50) solve")
    args = ap.parse_args()
    if args.mode == "passes":
        return run_passes(args)
    if args.mode == "koch":
        return run_koch(args)
    if args.mode == "adjoint":
        return run_adjoint(args)
    if args.mode == "nop":
        return run_nop(args)
    if args.mode == "lu":
        return run_lu(args)
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())

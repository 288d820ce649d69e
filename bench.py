"""Benchmark: global-matrix build throughput of the pede data loop.

One step = one data loop (local fits of every record, rejection decisions,
Schur-complement updates accumulated into the mpbits-sparse global matrix
and the gradient) over the barrel workload: 12-layer barrel, 5000 modules x
6 rigid-body parameters = 30000 global parameters, 2,000,000 linearised
helix tracks with 5 local parameters and 12 two-dimensional hits (72 global
parameters per record), 18 constraints.  Synthetic, seeded data of those
sizes (there is no public dataset for it).

value  : records/s with the records resident in HBM (device-timed loop)
e2e    : records/s through the C-ABI from pinned host buffers: every step
         uploads the records (mpgpu_upload_records) and runs mpgpu_loopbf
         with the global parameters in and the gradient/counts out
--impl reference: the CPU oracle (FP64 C restatement of loopbf + the
         sparse update) on all host cores over a bounded record sample.

Launch: python bench.py [--gpus N --steps K --warmup W]; for N > 1 through
torchrun, each rank processing its own replica (weak scaling, no exchange).
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "tests"))


def _load_pkg():
    import importlib.util
    spec = importlib.util.spec_from_file_location(
        "millepede_ii_gb300_mpgpu", os.path.join(ROOT, "millepede-ii_gb300", "mpgpu.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules["millepede_ii_gb300_mpgpu"] = mod
    spec.loader.exec_module(mod)
    return mod


def dist_setup(ngpus):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist
        backend = "nccl"
        try:
            import torch
            torch.cuda.set_device(local)
        except Exception:
            backend = "gloo"
        dist.init_process_group(backend=backend)
        pg = dist
    return rank, world, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if pg.get_backend() == "nccl" else "cpu")
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if pg.get_backend() == "nccl" else "cpu")
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        # raw samples in MPGPU_CLOCK_DIR when given (kept for inspection),
        # else in the temporary directory; the summary goes into the line
        base = os.environ.get("MPGPU_CLOCK_DIR") or tempfile.gettempdir()
        self.path = os.path.join(base, f"clocks_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        out = {"sm_mhz": None, "sm_max_mhz": None, "reasons": []}
        if self.proc is None:
            return out
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sms, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sms.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if sms:
            out = {"sm_mhz": statistics.median(sms), "sm_max_mhz": mx, "reasons": sorted(reasons),
                   "samples": len(sms)}
        return out


def flops_per_record(nmeas, nloc, ng, nalg):
    """Algorithmic FP64 flops of one record's local fit and update."""
    c_solve = nloc ** 3
    return 2 * (nmeas * (nloc + nloc * (nloc + 1) // 2) + c_solve + nmeas * ng * (ng + 1) // 2
                + nmeas * ng * nloc + nalg * nloc * nloc + nloc * nalg * (nalg + 1) // 2)


def record_shape(d):
    """(nmeas, nloc, ng, nalg) of the uniform barrel records."""
    a, b = int(d["recPtr"][0]), int(d["recPtr"][1])
    ii = d["inder"][a:b]
    zeros = np.flatnonzero(ii == 0)
    nmeas = (len(zeros) - 1) // 2
    sl, sg = zeros[1], zeros[2]
    nloc = int(ii[sl + 1:sg].max())
    nxt = zeros[3] if len(zeros) > 3 else b - a
    ng = int(nxt - sg - 1)
    nalg = 6 * 12
    return nmeas, nloc, ng, nalg


def dense_solve_measure(mp, local, ncon=120, nmod=2000, ntracks=400_000, sqminl=False, cond=0.0,
                        skip_slow=False):
    """Dense solve of the scaled telescope (10 layers x nmod modules = 20,000
    globals, packed FP64 matrix from the data loop, ncon constraints: the
    generator's 2 weak-mode constraints plus seeded sparse random ones, all
    eliminated by QL in FP64): the reference-structured FP64 Cholesky
    (metsol 3), the blocked FP64 Cholesky (32) and the tensor-core 3xTF32
    Cholesky (31), the latter two refined by FP64 CG to a relative residual
    of 1e-13.  The inversions from the blocked factors (metsol 12 FP64, 11
    tensor-core; with sqminl, also the reference-structured Gauss-Jordan,
    metsol 1) give the parameter errors."""
    cfg = mp.gen_config("telescope_dense", ntracks=ntracks, seed=4)
    cfg.nmod = nmod
    d = mp.generate(cfg)
    H = mp.HostStructure(d, mreqenf=5, sparse=False)
    A0 = mp.constraint_matrix(d, H)
    rng = np.random.default_rng(11)
    reg = 0.0
    if cond:
        # weak modes partly constrained: the sum of the shifts is fixed, the
        # shear (shift proportional to z) is left to a small diagonal
        # regularisation of 1/cond times the largest diagonal element, and
        # the other constraints sum to zero inside one layer, so they do not
        # touch either weak mode; cond(reduced matrix) is then about cond
        A0 = A0[:1]
        layer = (H.labels[H.varIndex > 0] - 1) // nmod
        extra = np.zeros((ncon - 1, H.nVar))
        for k in range(extra.shape[0]):
            pool = np.flatnonzero(layer == rng.integers(0, 10))
            idx = rng.choice(pool, 64, replace=False)
            c = rng.normal(size=64)
            extra[k, idx] = c - c.mean()
    else:
        extra = np.zeros((ncon - A0.shape[0], H.nVar))
        for k in range(extra.shape[0]):
            idx = rng.choice(H.nVar, 64, replace=False)
            extra[k, idx] = rng.normal(size=64)
    A = np.vstack([A0, extra])
    res = {}
    forms = (32, 31) if skip_slow else (32, 31, 3, 12, 11) + ((1,) if sqminl else ())
    for metsol in forms:
        ctx = mp.Context(device=local)
        ctx.set_layout(H, 1)
        ctx.set_constraints(A)
        ctx.upload(H)
        ctx.loopbf(np.zeros(H.nTotal))
        if cond:
            dg = ctx.matrix_diagonal()
            reg = float(np.max(dg)) / cond
            iv = np.arange(1, H.nVar + 1, dtype=np.int32)
            ctx.mupdat(iv, iv, np.full(H.nVar, reg))
        inv = metsol in (1, 11, 12)
        corr, err, info = ctx.solve(metsol, consResiduals=np.zeros(A.shape[0]), rtol=1e-13, itnlim=2000,
                                    errors=inv)
        res[metsol] = (corr, info.ms, info.itn, info.istop, info.msFactor, info.msRefine, err, info.msInverse,
                       info.dxRel)
        ctx.close()
    ref = res[32][0]
    # CPU baseline: the oracle's chdec2 (pede's method cholesky,
    # mpnum.f90:891-987, one core) on the same telescope with 2,000 globals
    # (200 modules per layer, tracks in proportion), scaled by (n / 2000)^3
    import oracle_ref as orc
    nsub = 2000
    cfg_s = mp.gen_config("telescope_dense", ntracks=max(ntracks * 200 // nmod, 1000), seed=4)
    cfg_s.nmod = 200
    d_s = mp.generate(cfg_s)
    H_s = mp.HostStructure(d_s, mreqenf=5, sparse=False)
    nsub = H_s.nVar
    with mp.Context(device=local) as ctx:
        ctx.set_layout(H_s, 1)
        ctx.upload(H_s)
        ctx.loopbf(np.zeros(H_s.nTotal))
        g = np.ascontiguousarray(ctx.matrix())
    nrank, evmax, evmin = C.c_int32(), C.c_double(), C.c_double()
    t0 = time.perf_counter()
    orc.lib().mpref_chdec2(orc.ptr(g, orc.f64p), C.c_int32(nsub), C.byref(nrank), C.byref(evmax), C.byref(evmin))
    cpu_s = time.perf_counter() - t0
    cpu_est_ms = cpu_s * 1e3 * (H.nVar / nsub) ** 3

    def rel(x, r=ref):
        return float(np.max(np.abs(x - r)) / np.max(np.abs(r)))

    def relerr(e, r):
        v = np.abs(r) > 0
        return float(np.max(np.abs(e[v] - r[v]) / np.abs(r[v])))
    out = {"n": int(H.nVar), "ncon": int(A.shape[0]), "nfit": int(H.nVar - A.shape[0]),
           "matrix": "scaled telescope, packed FP64 from the data loop" +
                     (f", shear weak mode regularised by max(diag)/{cond:.0e}" if cond else ""),
           "regularisation": reg,
           "ms_fp64_blocked": res[32][1], "ms_mixed_tf32x3": res[31][1],
           "speedup_mixed_vs_fp64_blocked": res[32][1] / res[31][1],
           "ms_factor_fp64_blocked": res[32][4], "ms_factor_mixed": res[31][4],
           "ms_refine_fp64_blocked": res[32][5], "ms_refine_mixed": res[31][5],
           "factor_speedup_mixed_vs_fp64_blocked": res[32][4] / max(res[31][4], 1e-9),
           "cg_iterations_mixed": res[31][2], "cg_iterations_fp64": res[32][2],
           "last_rel_correction_mixed": res[31][8], "last_rel_correction_fp64": res[32][8],
           "rel_err_mixed_vs_fp64": rel(res[31][0]),
           "converged": bool(res[31][3] == 1 and res[32][3] == 1),
           "cpu_baseline": {"value": cpu_est_ms, "unit": "ms", "cores": 1, "kind": "port",
                            "sample": f"oracle chdec2 of the same telescope with {nsub} globals "
                                      f"({cpu_s:.2f} s), scaled by (n/{nsub})^3"},
           "speedup_mixed_vs_cpu_chdec2_estimate": cpu_est_ms / res[31][1]}
    if 3 in res:
        out["ms_fp64_chdec2"] = res[3][1]
        out["speedup_mixed_vs_fp64_chdec2"] = res[3][1] / res[31][1]
        out["rel_err_chdec2_vs_fp64_blocked"] = rel(res[3][0])
    if 12 in res:
        out["inversion"] = {
               "ms_fp64_blocked": res[12][1], "ms_mixed_tf32x3": res[11][1],
               "ms_inverse_fp64_blocked": res[12][7], "ms_inverse_mixed": res[11][7],
               "rel_err_parameters_mixed_vs_fp64": rel(res[11][0], res[12][0]),
               "rel_err_errors_mixed_vs_fp64": relerr(res[11][6], res[12][6]),
               "refinement_steps_mixed": res[11][2], "refinement_steps_fp64": res[12][2],
               "note": "errors of the tensor-core inverse are not refined: about 1e-7 x cond"}
    if 1 in res:
        out["inversion"]["ms_sqminl"] = res[1][1]
        out["inversion"]["rel_err_errors_fp64_blocked_vs_sqminl"] = relerr(res[12][6], res[1][6])
        out["inversion"]["rel_err_parameters_fp64_blocked_vs_sqminl"] = rel(res[12][0], res[1][0])
    return out


def whole_job_measure(mp, d, local, cpu_loop_rate, cpu_minres_ms, pinned=None):
    """The 2M-record barrel as a whole job through mpgpu_pede_run: structure
    passes on the device, mpbits-sparse storage, 18 constraints eliminated,
    three solutions by MINRES with the diagonal preconditioner to a relative
    residual of 1e-12, outlier down-weighting in the second and third data
    loop (lhuber 2), chi2 cuts 30 then 6.  Wall time of the call; the CPU
    estimate is three loops at the measured CPU loop rate plus the MINRES
    iterations at the measured CPU time per iteration.  The records come
    from page-locked host buffers (recPtr and glder of the e2e steps, the
    raw labels copied into one more)."""
    raw = None
    if pinned is not None:
        raw = mp.PinnedArray(np.asarray(d["inder"]))
        d = dict(d, recPtr=pinned[0].a, inder=raw.a, glder=pinned[2].a)
    jd = mp.JobData(d, metsol=4, matsto=2, mitera=3, lhuber=2, chicut=30.0, chirem=6.0, mrestl=1e-12,
                    itnlim=6000, mreqenf=25, structDevice=1)
    t0 = time.perf_counter()
    rc = mp.run_job(jd)
    wall = time.perf_counter() - t0
    if raw is not None:
        raw.free()
    nrec = len(d["recPtr"]) - 1
    out = {"records": nrec, "rc": int(rc), "wall_s": wall, "solutions": 3, "metsol": 4, "rtol": 1e-12,
           "nrej_last": [int(v) for v in jd.res.nrej], "minres_iterations_last": int(jd.res.minresItn),
           "minres_istop_last": int(jd.res.minresIstop), "ms_loop_last": jd.res.msBuild,
           "ms_structure": jd.res.msStructure, "ms_upload": jd.res.msUpload, "ms_loops": jd.res.msLoops,
           "ms_solves": jd.res.msSolves, "ms_host_between": jd.res.msHostIter,
           "ms_solve_last": jd.res.msSolve}
    if cpu_loop_rate and cpu_minres_ms:
        est = 3 * nrec / cpu_loop_rate + 3 * jd.res.minresItn * cpu_minres_ms * 1e-3
        out["cpu_estimate_s"] = est
        out["cpu_estimate"] = ("3 data loops at the oracle's measured loop rate + 3 x the last solve's MINRES "
                               "iterations at the oracle's measured time per iteration (all host cores)")
        out["speedup_vs_cpu_estimate"] = est / wall
    return out


def minres_measure(mp, local, iters=300, cpu_iters=20, ncores=1):
    """MINRES on the sparse barrel (30,000 tracks: 30,000 globals, 6.1M
    stored elements, 18 constraints eliminated by QL): device time per
    iteration (a fixed number of iterations, rtol below reach) with the
    diagonal and the band-6 preconditioner, set-up time apart; the FP64
    bound of the sparse product (2 FMAs per stored off-diagonal element, 2
    FMAs per SM per clock on 152 SMs); and the oracle's MINRES on the host
    cores for cpu_iters iterations on the same matrix."""
    import ctypes as C
    import oracle_ref as orc
    d = mp.generate(mp.gen_config("barrel", ntracks=30000, seed=4))
    H = mp.HostStructure(d, mreqenf=5, sparse=True)
    A = mp.constraint_matrix(d, H)
    ctx = mp.Context(device=local)
    ctx.set_layout(H, 2)
    ctx.set_constraints(A)
    ctx.upload(H)
    lb = ctx.loopbf(np.zeros(H.nTotal))
    M = ctx.matrix()
    out = {"n": int(H.nVar), "ncon": int(A.shape[0]), "nmat": int(len(M)), "iterations": iters}
    for mb in (0, 6):
        ctx.set_preconditioner(mb)
        ctx.solve(4, consResiduals=np.zeros(A.shape[0]), rtol=1e-30, itnlim=16)
        _, _, info = ctx.solve(4, consResiduals=np.zeros(A.shape[0]), rtol=1e-30, itnlim=iters)
        key = "diagonal" if mb == 0 else "band6"
        out[f"ms_per_iteration_{key}"] = (info.ms - info.msFactor) / max(info.itn, 1)
        out[f"ms_setup_{key}"] = info.msFactor
    ctx.close()
    fmas = 2 * (len(M) - H.nVar) + H.nVar
    out["spmv_fp64_bound_us"] = fmas / (2 * 152 * 2.07e9) * 1e6
    # algorithmic bytes per iteration: the stored matrix and its column
    # words once, about ten vectors of N doubles
    try:
        hbm = float(json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))).get("hbm_gbs", 6800.0))
        src = "MEASURED_PEAKS.json hbm_gbs"
    except (OSError, ValueError):
        hbm, src = 6800.0, "fallback"
    nbytes = 8 * len(M) + 4 * int(H.ncolw) + 80 * H.nVar
    gbs = nbytes / (out["ms_per_iteration_diagonal"] * 1e-3) / 1e9
    out["roofline_diagonal"] = {"bytes_per_iteration": nbytes, "achieved_gbs": gbs, "peak_gbs": hbm,
                                "frac": gbs / hbm, "peak_source": src,
                                "hbm_bound_us": nbytes / (hbm * 1e9) * 1e6,
                                "binding": "fp64" if out["spmv_fp64_bound_us"] > nbytes / (hbm * 1e3) else "hbm"}
    # the oracle's MINRES (diagonal) on one host core, same matrix and rhs
    L = orc.lib()
    f64p, i32p, i64p = C.POINTER(C.c_double), C.POINTER(C.c_int32), C.POINTER(C.c_int64)
    L.mpref_ql_create.restype = C.c_void_p
    Ac = np.ascontiguousarray(A)
    q = L.mpref_ql_create(C.c_int32(H.nVar), C.c_int32(A.shape[0]), Ac.ctypes.data_as(f64p))
    b = lb["gvec"].copy()
    L.mpref_ql_mlq(C.c_void_p(q), b.ctypes.data_as(f64p), C.c_int32(1))
    x = np.zeros(H.nVar)
    itn, nrkd = C.c_int32(), C.c_int32()
    off = np.ascontiguousarray(H.offsets, np.int64)
    col = np.ascontiguousarray(H.columns, np.int32)
    L.mpref_set_threads(C.c_int32(ncores))
    t0 = time.perf_counter()
    L.mpref_minres_precond(C.c_int32(0), C.c_int32(2), C.c_int32(H.nVar), C.c_int32(H.nG),
                           H.aig.ctypes.data_as(i32p), off.ctypes.data_as(i64p), col.ctypes.data_as(i32p),
                           M.ctypes.data_as(f64p), C.c_void_p(q), b.ctypes.data_as(f64p), x.ctypes.data_as(f64p),
                           C.c_double(1e-30), C.c_int32(cpu_iters), C.c_int32(0), C.c_int32(0), C.byref(itn),
                           C.byref(nrkd))
    cpu_s = time.perf_counter() - t0
    L.mpref_set_threads(C.c_int32(1))
    L.mpref_ql_destroy(C.c_void_p(q))
    out["cpu_baseline"] = {"ms_per_iteration": cpu_s * 1e3 / max(itn.value, 1), "cores": ncores, "kind": "port",
                           "sample": f"{itn.value} iterations including the preconditioner set-up"}
    out["speedup_vs_cpu_diagonal"] = out["cpu_baseline"]["ms_per_iteration"] / out["ms_per_iteration_diagonal"]
    return out


def serve_measure(mp, local, njobs=24, rate=8.0, nmin=500, nmax=20000, rmin=10_000, rmax=200_000):
    """Stream of alignment jobs through the serving loop: Poisson arrivals at
    `rate` per second; per job (seed 1000 + job) a telescope with globals
    log-uniform in [nmin, nmax] and records log-uniform in [rmin, rmax],
    3 iterations with outlier down-weighting, dense solve (tensor-core
    factor + FP64 CG).  The same jobs, same arrivals, one at a time with the
    FP64 blocked dense solve, give the plain-form comparison."""
    rng = np.random.default_rng(7)
    specs = []
    for k in range(njobs):
        n = int(np.exp(rng.uniform(np.log(nmin), np.log(nmax))))
        nrec = int(np.exp(rng.uniform(np.log(rmin), np.log(rmax))))
        cfg = mp.gen_config("telescope", ntracks=nrec, seed=1000 + k)
        cfg.nmod = max(n // 10, 5)
        specs.append(mp.generate(cfg))
    arrivals = np.cumsum(rng.exponential(1.0 / rate, njobs))

    def run(metsol, active):
        jds = [mp.JobData(d, metsol=metsol, matsto=1, mitera=3, lhuber=2, chicut=30.0, chirem=6.0,
                          mreqenf=5) for d in specs]
        with mp.Server(device=local, max_active=active) as srv:
            t0 = time.perf_counter()
            tickets = []
            for jd, ta in zip(jds, arrivals):
                dt = ta - (time.perf_counter() - t0)
                if dt > 0:
                    time.sleep(dt)
                tickets.append(srv.submit(jd))
            out = [srv.wait(t, timeout_ms=1.8e6) for t in tickets]
            span = time.perf_counter() - t0
        lat = np.array([o[1] for o in out])
        return {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                "jobs_per_s": njobs / span, "ok": all(o[0] == 0 for o in out)}, jds
    served, jds = run(31, 4)
    plain, jdp = run(32, 1)
    # one solution per job (no iteration): mixed against FP64 on the same
    # matrix; the iterated jobs below differ more because each Gauss-Newton
    # step amplifies the gradient's rounding noise by cond(A), for any form
    single = []
    for d in specs:
        p = {}
        for ms in (31, 32):
            jd = mp.JobData(d, metsol=ms, matsto=1, mitera=1, mreqenf=5)
            assert mp.run_job(jd) == 0
            p[ms] = jd
        single.append(float(np.max(np.abs(p[31].parameters()[1] - p[32].parameters()[1])) /
                            max(float(np.max(np.abs(p[32].parameters()[1]))), 1e-300)))
    diffs = [float(np.max(np.abs(a.parameters()[1] - b.parameters()[1])) /
                   max(float(np.max(np.abs(b.parameters()[1]))), 1e-300)) for a, b in zip(jds, jdp)]
    steps_m = [int(a.res.minresItn) for a in jds]
    steps_f = [int(b.res.minresItn) for b in jdp]
    return {"jobs": njobs, "arrival_rate_per_s": rate, "globals": [nmin, nmax], "records": [rmin, rmax],
            "iterations": 3, "served_concurrent_mixed": served, "one_at_a_time_fp64": plain,
            "max_rel_diff_parameters_single_solve": max(single), "tolerance": 1e-10,
            "single_solve_within_tolerance": bool(max(single) <= 1e-10),
            "max_rel_diff_parameters_iterated": max(diffs), "rel_diff_parameters_iterated_per_job": diffs,
            "refinement_steps_last_solve_mixed": steps_m, "refinement_steps_last_solve_fp64": steps_f}


def sample_of(d, nsample):
    rp = d["recPtr"][:nsample + 1]
    return dict(recPtr=rp, inder=d["inder"][:rp[-1]], glder=d["glder"][:rp[-1]])


SERVE_SPEC_STEER = dict(matsto=1, mitera=3, lhuber=2, chicut=30.0, chirem=6.0, mreqenf=5)


def serve_spec_plan(njobs, rate=4.0, nmin=500, nmax=40000, rmin=10_000, rmax=1_000_000):
    """Per job (model, globals drawn, records, constraints) and the Poisson
    arrival times of the serving stream (seeded)."""
    rng = np.random.default_rng(29)
    specs = []
    for k in range(njobs):
        n = int(np.exp(rng.uniform(np.log(nmin), np.log(nmax))))
        nrec = int(np.exp(rng.uniform(np.log(rmin), np.log(rmax))))
        kind = "barrel" if rng.random() < 0.5 else "brokenlines"
        specs.append((kind, n, nrec, int(rng.integers(6, 61))))
    return specs, np.cumsum(rng.exponential(1.0 / rate, njobs))


def serve_spec_job(mp, specs, k):
    """Records and constraints of job k of the serving stream (seed 1000 + k):
    the barrel with n/6 modules, helix or broken-line (4-28 hits) tracks,
    the model's weak-mode constraints plus seeded sparse ones up to the
    drawn count; returns (data, constraints, number of detector labels)."""
    kind, n, nrec, ncon = specs[k]
    cfg = mp.gen_config(kind, ntracks=nrec, seed=1000 + k)
    cfg.nmod = max(n // 6, 1)
    cfg.threads = 6   # tracks on six host threads, each from its own stream
    if kind == "brokenlines":
        cfg.maxHits = 28
    d = mp.generate(cfg)
    crng = np.random.default_rng(5000 + k)
    # the detector's labels 1..6 nmod (a label no record carries is dropped
    # from its constraint by the job driver)
    labels = np.arange(1, len(d["truth"]) + 1, dtype=np.int32)
    cs, cl, cc = list(d["conStart"]), list(d["conLabel"]), list(d["conCoef"])
    for _ in range(max(0, ncon - d["ncon"])):
        pick = crng.choice(labels, min(64, len(labels)), replace=False)
        c = crng.normal(size=len(pick))
        cl += [int(x) for x in pick]
        cc += [float(x) for x in c - c.mean()]
        cs.append(len(cl))
    return d, (np.array(cs, np.int32), np.array(cl, np.int32), np.array(cc)), len(labels)


def serve_spec_measure(mp, local, njobs=256, rate=4.0, nmin=500, nmax=40000, rmin=10_000, rmax=1_000_000,
                       fp64="all", budget_gb=150, gen_threads=2, lookahead=12, max_active=4):
    """The stream of alignment jobs at its specified shape: njobs jobs with
    Poisson arrivals at `rate` per second, each generated from its own seed
    (1000 + job) with the barrel detector model, as helix tracks (12 hits,
    nloc 5) or broken lines (4-28 hits, nloc 12-60), globals log-uniform in
    [nmin, nmax] (the barrel's smallest layout has 1,728), records
    log-uniform in [rmin, rmax], 6-60 linear constraints (the 18 weak-mode
    constraints of the barrel plus seeded sparse ones), 3 iterations with
    outlier down-weighting, dense tensor-core Cholesky + FP64 refinement
    (every size is at most 40,000), admitted by device footprint against
    budget_gb, max_active jobs active.  Jobs are generated ahead of their arrival
    (two at a time, each on six host threads; at most `lookahead` in memory).  The same jobs
    then run one at a time with the FP64 blocked solve (fp64 "all", or
    "every8" for every 8th job), whose latencies under the same arrivals are
    those of a first-come-first-served queue over the measured service
    times."""
    import threading
    from concurrent.futures import ThreadPoolExecutor
    specs, arrivals = serve_spec_plan(njobs, rate, nmin, nmax, rmin, rmax)
    steer = SERVE_SPEC_STEER

    def make(k):
        return serve_spec_job(mp, specs, k)

    errors = []

    def phases(jd):
        r = jd.res
        return dict(structure_ms=r.msStructure, upload_ms=r.msUpload, loops_ms=r.msLoops, solves_ms=r.msSolves,
                    host_iter_ms=r.msHostIter, job_ms=r.msJob, nrej=int(sum(r.nrej)))

    def stream(metsol, serve):
        """(per-job records, span): served concurrently at the arrival times,
        or one at a time back to back (service times)."""
        out = [None] * njobs
        pool = ThreadPoolExecutor(gen_threads)
        fut = {}
        nxt = 0

        def ahead(upto):
            nonlocal nxt
            while nxt < min(upto, njobs):
                fut[nxt] = pool.submit(make, nxt)
                nxt += 1
        ahead(lookahead)
        keep = set(range(0, njobs, 8)) if fp64 == "every8" else set(range(njobs))
        if serve:
            srv = mp.Server(device=local, max_active=max_active, budget_bytes=budget_gb << 30)
            tickets = []
            done = threading.Event()

            def waiter():
                for k in range(njobs):
                    while len(tickets) <= k:
                        time.sleep(0.005)
                    t, jd, lag, nglob = tickets[k]
                    rc, lat, q, b = srv.wait(t, timeout_ms=3.6e6)
                    out[k] = dict(rc=int(rc), lat_ms=lat, queue_ms=q, bytes=int(b), lag_ms=lag, n=int(jd.res.nVar),
                                  globals=nglob, nrec=int(jd.job.nrec), ncon=int(jd.job.ncon),
                                  cg_last=int(jd.res.minresItn), **phases(jd),
                                  par=jd.parameters()[1] if k in keep else None)
                    tickets[k] = None   # the job's host arrays go
                    del jd
                done.set()
            wt = threading.Thread(target=waiter)
            wt.start()
            t0 = time.perf_counter()
            for k in range(njobs):
                d, con, nglob = fut.pop(k).result()
                ahead(k + 1 + lookahead)
                jd = mp.JobData(d, constraints=con, metsol=metsol, **steer)
                del d
                now = time.perf_counter() - t0
                if arrivals[k] > now:
                    time.sleep(arrivals[k] - now)
                lag = max(0.0, (time.perf_counter() - t0) - arrivals[k]) * 1e3
                tickets.append((srv.submit(jd), jd, lag, nglob))
            done.wait()
            span = time.perf_counter() - t0
            wt.join()
            errors.append(srv.last_error())
            srv.close()
        else:
            span = 0.0
            for k in range(njobs):
                d, con, nglob = fut.pop(k).result()
                ahead(k + 1 + lookahead)
                if k not in keep:
                    continue
                jd = mp.JobData(d, constraints=con, metsol=metsol, **steer)
                del d
                # the serving workers' fixed 8 GiB update staging (the same
                # chunking, so the same loop sums as in the served stream)
                ctx = mp.Context(device=local, staging_bytes=8 << 30)
                t1 = time.perf_counter()
                rc = mp.run_job(jd, ctx)
                ms = (time.perf_counter() - t1) * 1e3
                ctx.close()
                span += ms * 1e-3
                out[k] = dict(rc=int(rc), service_ms=ms, n=int(jd.res.nVar), cg_last=int(jd.res.minresItn),
                              **phases(jd), par=jd.parameters()[1])
                if rc:
                    out[k]["error"] = ctx.last_error()
        pool.shutdown()
        return out, span

    served, span = stream(31, True)
    lat = np.array([o["lat_ms"] for o in served])
    ok = [o["rc"] == 0 for o in served]
    res = {"jobs": njobs, "arrival_rate_per_s": rate, "globals_drawn": [nmin, nmax],
           "globals_actual": [min(o["n"] for o in served), max(o["n"] for o in served)],
           "records": [min(o["nrec"] for o in served), max(o["nrec"] for o in served)],
           "models": {m: sum(1 for s in specs if s[0] == m) for m in ("barrel", "brokenlines")},
           "constraints": [min(o["ncon"] for o in served), max(o["ncon"] for o in served)],
           "iterations": 3, "budget_gb": budget_gb, "max_active": max_active, "solve": "metsol 31 (tensor-core factor, "
           "FP64 CG refinement, factor kept across the job's iterations)",
           "served_mixed": {"p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                            "jobs_per_s": njobs / span, "span_s": span, "ok": all(ok),
                            "rc": sorted(set(o["rc"] for o in served)),
                            "queue_p50_ms": float(np.percentile([o["queue_ms"] for o in served], 50)),
                            "arrival_lag_max_ms": max(o["lag_ms"] for o in served),
                            "last_error": errors[0] if errors else ""}}
    res["per_job"] = [{k: (round(v, 3) if isinstance(v, float) else v) for k, v in o.items() if k != "par"}
                      for o in served]
    if fp64:
        plain, busy = stream(32, False)
        idx = [k for k in range(njobs) if plain[k] is not None]
        svc = np.array([plain[k]["service_ms"] for k in idx])
        entry = {"jobs": len(idx), "service_p50_ms": float(np.percentile(svc, 50)),
                 "service_p99_ms": float(np.percentile(svc, 99)), "busy_s": busy,
                 "ok": all(plain[k]["rc"] == 0 for k in idx)}
        if len(idx) == njobs:
            # first-come-first-served single server over the measured service
            # times at the same arrival times
            fin, lq = 0.0, []
            for k in range(njobs):
                start = max(arrivals[k] * 1e3, fin)
                fin = start + svc[k]
                lq.append(fin - arrivals[k] * 1e3)
            entry.update({"p50_ms": float(np.percentile(lq, 50)), "p99_ms": float(np.percentile(lq, 99)),
                          "jobs_per_s": njobs / (max(fin * 1e-3, arrivals[-1]))})
        res["one_at_a_time_fp64"] = entry
        diffs = [float(np.max(np.abs(served[k]["par"] - plain[k]["par"])) /
                       max(float(np.max(np.abs(plain[k]["par"]))), 1e-300))
                 for k in idx if served[k]["rc"] == 0 and plain[k]["rc"] == 0]
        res["max_rel_diff_parameters_iterated"] = max(diffs) if diffs else None
        res["median_rel_diff_parameters_iterated"] = float(np.median(diffs)) if diffs else None
        for k in idx:
            res["per_job"][k]["fp64_service_ms"] = round(plain[k]["service_ms"], 3)
            res["per_job"][k]["fp64_rc"] = plain[k]["rc"]
            res["per_job"][k]["fp64_nrej"] = plain[k]["nrej"]
            if plain[k]["rc"]:
                res["per_job"][k]["fp64_error"] = plain[k].get("error", "")
    return res


def cpu_reference(d, nsample, nthreads, steps=1, keep=False):
    """CPU oracle (loopbf restatement, OpenMP) on the first nsample records;
    with keep, also the oracle's structure and the output of the last step."""
    import oracle_ref as orc
    S = orc.Structure(sample_of(d, nsample), mreqenf=1)
    gpar = np.zeros(S.nTotal)
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        o = S.loopbf(gpar, matsto=2, nthreads=nthreads)
        times.append(time.perf_counter() - t0)
        assert o["rc"] == 0
    if keep:
        return nsample / statistics.median(times), times, S, o
    return nsample / statistics.median(times), times


def bench_parity(mp, device, d, nsample, S, o):
    """The device data loop on the records the CPU leg timed (the first
    nsample records of the workload, their own label table and mpbits
    structure), against the oracle's output of that leg: tables and record
    decisions bit for bit, matrix, vector and chi2 within 1e-12 relative."""
    sub = sample_of(d, nsample)
    H = mp.HostStructure(sub, mreqenf=1)
    same_tables = bool(np.array_equal(H.labels, S.labels) and np.array_equal(H.varIndex, S.varIndex)
                       and np.array_equal(H.aig, S.aig) and np.array_equal(H.offsets, S.offsets)
                       and np.array_equal(H.columns[:H.ncolw], S.columns[:S.ncolw]))
    with mp.Context(device=device) as ctx:
        ctx.set_layout(H, 2)
        ctx.upload(H)
        g = ctx.loopbf(np.zeros(H.nTotal))
        M = ctx.matrix()
        st = ctx.status()

    def rel(a, b):
        return float(np.max(np.abs(a - b)) / max(float(np.max(np.abs(b))), 1e-300))
    out = {"records": nsample, "tables_equal": same_tables,
           "status_equal": bool(np.array_equal(st, o["status"])),
           "nrej_equal": bool(list(g["nrej"]) == list(o["nrej"])), "nrej": list(g["nrej"]),
           "matrix_rel": rel(M, o["matD"]), "vector_rel": rel(g["gvec"], o["gvec"]),
           "counts_equal": bool(np.array_equal(g["gcnt"], o["gcnt"])),
           "chi2_rel": abs(g["chi2"] - o["chi2"]) / max(abs(o["chi2"]), 1e-300)}
    out["ok"] = bool(out["tables_equal"] and out["status_equal"] and out["nrej_equal"] and out["counts_equal"]
                     and out["matrix_rel"] <= 1e-12 and out["vector_rel"] <= 1e-12)
    return out


def brokenlines_measure(mp, device, nrec, ncores, steps=2):
    """The uneven-record workload (broken-line tracks on the barrel, 4-40
    hits, nloc 8-84, nalg 24-240; sparse storage): device data loops with
    the records in fit size classes (tuned warps per CTA), with one launch
    sized for the largest record, and with one record per CTA; the CPU
    oracle on a sample; then the same records as a whole job solved by the
    tensor-core Cholesky (metsol 31, full storage, 18 constraints
    eliminated, one iteration).  The tracks are generated on all host
    threads, each from its own seeded stream."""
    cfg = mp.gen_config("brokenlines", ntracks=nrec, seed=3)
    cfg.threads = ncores
    d = mp.generate(cfg)
    H = mp.HostStructure(d, mreqenf=25)
    gpar = np.zeros(H.nTotal)
    out = {"records": nrec, "hits": [4, 40], "nloc": [8, 84]}
    forms = (("size_classes", 0), ("one_launch_largest_record", mp.FLAG_NO_BUCKETS),
             ("one_record_per_block", mp.FLAG_ONE_RECORD_PER_BLOCK))
    for name, flags in forms:
        with mp.Context(device=device, flags=flags) as ctx:
            ctx.set_layout(H, 2)
            ctx.upload(H)
            ctx.loopbf(gpar)
            ms, fit = [], []
            for _ in range(steps):
                r = ctx.loopbf(gpar)
                ms.append(r["msLoop"])
                fit.append(r["msFit"])
            cnt, wpc, tms = ctx.fit_buckets()
        e = {"records_per_s": nrec / (statistics.median(ms) * 1e-3), "ms_loop": ms, "ms_fit": fit}
        if flags == 0:
            e["class_records"] = cnt.tolist()
            e["class_warps_per_cta"] = wpc.tolist()
            e["class_tune_ms_1_2_4_8_warps"] = [[round(x, 3) for x in row] for row in tms.tolist()]
        out[name] = e
    base = out["one_record_per_block"]["records_per_s"]
    out["speedup_size_classes_vs_one_record_per_block"] = out["size_classes"]["records_per_s"] / base
    # the configuration's solve: method cholesky of the 30,000 globals, as
    # one job from page-locked host buffers with the structure passes on the
    # device (the records are copied once and kept for the data loop)
    pin = [mp.PinnedArray(np.asarray(d[k])) for k in ("recPtr", "inder", "glder")]
    dj = dict(d, recPtr=pin[0].a, inder=pin[1].a, glder=pin[2].a)
    jd = mp.JobData(dj, metsol=31, matsto=1, mitera=1, mreqenf=25, mrestl=1e-13, itnlim=2000,
                    structDevice=1)
    with mp.Context(device=device) as ctx:
        t0 = time.perf_counter()
        rc = mp.run_job(jd, ctx)
        wall = time.perf_counter() - t0
    r = jd.res
    out["cholesky_job"] = {"rc": int(rc), "metsol": 31, "globals": int(r.nVar), "constraints": 18,
                           "structure": "device passes, records from page-locked buffers",
                           "wall_s": wall, "ms_structure": r.msStructure, "ms_upload": r.msUpload,
                           "ms_loop": r.msLoops, "ms_solve": r.msSolves, "cg_iterations": int(r.minresItn)}
    del jd, dj
    for a in pin:
        a.free()
    nsample = min(5000, nrec)
    val, _ = cpu_reference(d, nsample, ncores, steps=1)
    out["cpu_baseline"] = {"value": val, "unit": "records/s", "cores": ncores, "kind": "port",
                           "sample": f"first {nsample} records, one sparse data loop"}
    return out


def structure_measure(mp, S, pinned, device, host_s, ncores):
    """loop1 + loop2 (label table, translation, entries, groups, mpbits) on
    the host (mpgpu_host_labels/translate/mpbits, all host threads) and on
    the device (mpgpu_loop1_device/loop2_device, the copy of the records from
    page-locked buffers included); the tables must be identical."""
    data = {"recPtr": pinned[0].a, "glder": pinned[2].a}
    # the raw (untranslated) words in the page-locked buffer for the device passes
    raw = mp.PinnedArray(np.asarray(S.rawInder))
    data["inder"] = raw.a
    times, same = [], True
    with mp.Context(device=device) as ctx:
        for _ in range(3):
            t0 = time.perf_counter()
            D = mp.DeviceStructure(ctx, data, mreqenf=25)
            times.append(time.perf_counter() - t0)
    for k in ("labels", "counter", "varIndex", "totGroup", "aig", "offsets"):
        same &= bool(np.array_equal(getattr(S, k), getattr(D, k)))
    same &= bool(np.array_equal(S.columns[:S.ncolw], D.columns[:D.ncolw]))
    raw.free()
    return {"records": len(S.recPtr) - 1, "host_s": host_s, "host_threads": ncores,
            "device_s": times, "device_s_median": statistics.median(times),
            "speedup": host_s / statistics.median(times), "tables_identical": same}


def profile_part(mp, part, ntracks, device, steps, mbandw=0):
    """One part of the path on a small case, for profilers: the record
    upload (barrel), the device structure passes (barrel) or the data loop
    of broken-line records (size classes, no tuning).  Each repeats `steps`
    times after one untimed pass.  `minres`: the barrel (seed 4) with its
    constraints, sparse matrix from one data loop, then two MINRES solves
    of `steps` iterations each (rtol below reach) with preconditioner
    `mbandw` (0 diagonal, > 0 band width)."""
    if part == "minres":
        d = mp.generate(mp.gen_config("barrel", ntracks=ntracks, seed=4))
        H = mp.HostStructure(d, mreqenf=5, sparse=True)
        A = mp.constraint_matrix(d, H)
        out = {"part": part, "n": int(H.nVar), "ncon": int(A.shape[0]), "mbandw": mbandw, "solves": []}
        with mp.Context(device=device) as ctx:
            ctx.set_layout(H, 2)
            ctx.set_constraints(A)
            ctx.upload(H)
            ctx.loopbf(np.zeros(H.nTotal))
            ctx.set_preconditioner(mbandw)
            for _ in range(2):
                _, _, info = ctx.solve(4, consResiduals=np.zeros(A.shape[0]), rtol=1e-30, itnlim=steps)
                out["solves"].append({"itn": info.itn, "ms": info.ms, "ms_setup": info.msFactor,
                                      "ms_per_iteration": (info.ms - info.msFactor) / max(info.itn, 1)})
        print(json.dumps(out))
        return
    kind = "brokenlines" if part == "brokenlines" else "barrel"
    d = mp.generate(mp.gen_config(kind, ntracks=ntracks, seed=3 if kind == "brokenlines" else 2))
    flags = mp.FLAG_NO_AUTOTUNE if part == "brokenlines" else 0
    out = {"part": part, "records": ntracks, "ms": []}
    with mp.Context(device=device, flags=flags) as ctx:
        if part == "structure":
            for k in range(steps + 1):
                t0 = time.perf_counter()
                mp.DeviceStructure(ctx, d, mreqenf=25)
                out["ms"].append(1e3 * (time.perf_counter() - t0))
        else:
            H = mp.HostStructure(d, mreqenf=25)
            ctx.set_layout(H, 2)
            for k in range(steps + 1):
                ctx.upload(H)
                if part == "upload":
                    out["ms"].append(ctx.upload_timing()[1])
                else:
                    out["ms"].append(ctx.loopbf(np.zeros(H.nTotal))["msLoop"])
    print(json.dumps(out))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--ntracks", type=int, default=2_000_000)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--cpu-sample", type=int, default=100_000)
    ap.add_argument("--profile", action="store_true", help="small run for profilers (no e2e/cpu)")
    ap.add_argument("--staging-mb", type=int, default=0, help="update staging buffer (0: default)")
    ap.add_argument("--dense-n", type=int, default=20000, help="globals of the dense-solve measurement (0: skip)")
    ap.add_argument("--dense-sqminl", action="store_true",
                    help="also time the reference-structured inversion (sqminl) in the dense measurement")
    ap.add_argument("--dense-cond", type=float, default=0.0,
                    help="dense measurement on the input with condition number about this (0: as generated)")
    ap.add_argument("--dense-only", action="store_true", help="only the dense measurement (with --dense-n)")
    ap.add_argument("--serve-spec", type=int, default=0,
                    help="only the serving stream at its specified shape with this many jobs (256)")
    ap.add_argument("--serve-fp64", default="all", choices=["all", "every8", ""],
                    help="--serve-spec: the one-at-a-time FP64 comparison over all jobs, every 8th, or none")
    ap.add_argument("--whole-job", type=int, default=1, help="time the barrel as a whole job (0: skip)")
    ap.add_argument("--minres-iters", type=int, default=300, help="iterations of the MINRES measurement (0: skip)")
    ap.add_argument("--mbandw", type=int, default=0, help="--part minres: preconditioner (0 diagonal, > 0 band width)")
    ap.add_argument("--serve-jobs", type=int, default=24, help="jobs of the serving measurement (0: skip)")
    ap.add_argument("--part", default="loop", choices=["loop", "upload", "structure", "brokenlines", "minres"],
                    help="with --profile: the part to run on --ntracks records (for profilers)")
    ap.add_argument("--brokenlines", type=int, default=1_000_000,
                    help="records of the uneven-record (broken-line) measurement (0: skip)")
    args = ap.parse_args()
    rank, world, local, pg = dist_setup(args.gpus)
    mp = _load_pkg()
    if args.profile and args.part != "loop":
        profile_part(mp, args.part, args.ntracks, local, args.steps, args.mbandw)
        return
    if args.serve_spec:
        if rank == 0:
            print(json.dumps(serve_spec_measure(mp, local, njobs=args.serve_spec, fp64=args.serve_fp64)))
        return
    if args.dense_only:
        if rank == 0:
            print(json.dumps(dense_solve_measure(mp, local, nmod=args.dense_n // 10, ntracks=20 * args.dense_n,
                                                 sqminl=args.dense_sqminl, cond=args.dense_cond,
                                                 skip_slow=args.dense_n > 40000)))
        return
    cfg = mp.gen_config("barrel", ntracks=args.ntracks, seed=2 + 1000 * rank)
    t0 = time.time()
    d = mp.generate(cfg)
    gen_s = time.time() - t0
    nrec = len(d["recPtr"]) - 1
    ncores = os.cpu_count() or 1
    base_cfg = {"workload": "barrel 12 layers, 5000 modules x 6 dof = 30000 globals, "
                            f"{args.ntracks} helix tracks x 12 2D hits (72 globals/record), "
                            "5 local params, 18 constraints, mpbits sparse storage",
                "records": nrec, "matsto": 2, "l2": "inputs (records, 7.5 GB) larger than L2",
                "parallelism": f"replicas x{world}"}

    if args.impl == "reference":
        if rank != 0:
            return
        nsample = min(args.cpu_sample, nrec)
        cpu_reference(d, min(nsample, 5000), ncores, steps=1)  # warm-up
        val, times = cpu_reference(d, nsample, ncores, steps=args.steps)
        line = {"metric": "records/s build", "value": val, "unit": "records/s", "n_gpus": 0,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": 1e3 * statistics.median(times), "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "impl": "reference", "config": dict(base_cfg, sample_records=nsample),
                "cpu_baseline": {"value": val, "unit": "records/s", "cores": ncores,
                                 "kind": "port",
                                 "sample": f"first {nsample} records of the workload, one data "
                                           "loop with sparse matrix build per step"},
                "e2e": {"value": val, "unit": "records/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    t0 = time.perf_counter()
    S = mp.HostStructure(d, mreqenf=25)
    host_struct_s = time.perf_counter() - t0
    A = mp.constraint_matrix(d, S)
    L = mp.lib()
    # the host record buffers in page-locked memory from the runtime (e2e
    # uploads read them); registering the numpy buffers instead gave uploads
    # that slowed down to pageable speed on some boxes after other GPU work
    pinned = [mp.PinnedArray(S.recPtr), mp.PinnedArray(S.tinder), mp.PinnedArray(S.glder)]
    S.recPtr, S.tinder, S.glder = pinned[0].a, pinned[1].a, pinned[2].a
    ctx = mp.Context(device=local, staging_bytes=args.staging_mb << 20)
    ctx.set_layout(S, 2)
    ctx.set_constraints(A)
    t0 = time.time()
    ctx.upload(S)
    upload_s = time.time() - t0
    gpar = np.zeros(S.nTotal)
    for _ in range(args.warmup):
        ctx.loopbf(gpar)
    clocks = ClockSampler(local)
    barrier(pg)
    clocks.start()
    t0 = time.perf_counter()
    ms_loop, ms_fit, ms_acc, launches = [], [], [], 0
    for _ in range(args.steps):
        r = ctx.loopbf(gpar)
        ms_loop.append(r["msLoop"])
        ms_fit.append(r["msFit"])
        ms_acc.append(r["msAccum"])
        launches += r["launches"]
    wall = time.perf_counter() - t0
    barrier(pg)
    clk = clocks.stop()
    dev_s = sum(ms_loop) * 1e-3
    dev_s_max = max_over_ranks(pg, dev_s)
    total_rec = sum_over_ranks(pg, float(nrec * args.steps))
    value = total_rec / dev_s_max
    ms_per_step = 1e3 * dev_s_max / args.steps
    nmeas, nloc, ng, nalg = record_shape(d)
    fpr = flops_per_record(nmeas, nloc, ng, nalg)
    fp64 = C.c_double()
    L.mpgpu_probe_fp64(C.c_int32(local), C.byref(fp64))
    fit_ms = statistics.median(ms_fit)
    achieved = fpr * nrec / (fit_ms * 1e-3) / 1e12
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    # accumulation kernel: staging read + block-row read/write of the matrix
    ngg = nalg * (nalg + 1) // 2
    acc_bytes = 8.0 * ngg * nrec + 16.0 * ctx.nmat
    acc_ms = statistics.median(ms_acc)
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    # DRAM traffic of k_fit per record from one ncu capture of the barrel
    # (dram__bytes_read.sum + dram__bytes_write.sum of a launch over a sample
    # of 45.5k records: 331 MB read, 961 MB written), scaled to this launch's
    # records; the writes are the block-major staging (21.1 KB per record)
    traffic_per_record = (331.5e6 + 961.3e6) / 45.5e3
    roof = {"bound": "fp64", "kernel": "k_fit (local fit + Schur update)",
            "achieved": achieved, "peak": fp64.value, "unit": "TFLOP/s",
            "frac": achieved / fp64.value if fp64.value else None,
            "traffic": traffic_per_record * nrec,
            "traffic_source": "ncu dram bytes of one k_fit launch on a 45.5k-record barrel sample, "
                              "scaled per record",
            "flops_per_record": fpr,
            "peak_source": "FP64 FMA throughput measured in this run (mpgpu_probe_fp64)",
            "accumulate": {"bound": "hbm", "achieved": acc_bytes / (acc_ms * 1e-3) / 1e9,
                           "peak": hbm_peak, "unit": "GB/s",
                           "frac": acc_bytes / (acc_ms * 1e-3) / 1e9 / hbm_peak,
                           "bytes_per_loop": acc_bytes,
                           "peak_source": "MEASURED_PEAKS.json hbm_gbs" if peaks else "fallback"}}
    line = {"metric": "records/s build", "value": value, "unit": "records/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": base_cfg, "roofline": roof, "clocks": clk,
            "gpu_launches": launches,
            "detail": {"ms_fit": fit_ms, "ms_accumulate": acc_ms, "wall_s": wall,
                       "nmat": ctx.nmat, "generate_s": gen_s, "upload_s": upload_s}}
    if not args.profile:
        # end to end through the C-ABI from pinned host buffers
        bi = S.tinder.nbytes + d["glder"].nbytes + d["recPtr"].nbytes + 8 * S.nTotal
        bo = 16 * S.nVar + 256
        barrier(pg)
        t0 = time.perf_counter()
        up_s, lp_s, up_dev = [], [], []
        for _ in range(args.e2e_steps):
            ta = time.perf_counter()
            ctx.upload(S)
            tb = time.perf_counter()
            ctx.loopbf(gpar)
            up_s.append(tb - ta)
            up_dev.append(ctx.upload_timing())
            lp_s.append(time.perf_counter() - tb)
        e2e_s = max_over_ranks(pg, time.perf_counter() - t0)
        line["e2e"] = {"value": total_rec / args.steps * args.e2e_steps / e2e_s,
                       "unit": "records/s", "h2d_bytes_per_step": bi, "d2h_bytes_per_step": bo,
                       "steps": args.e2e_steps, "upload_s": up_s, "loop_s": lp_s,
                       "upload_device_ms": up_dev, "pinned_buffers": len(pinned)}
        if rank == 0:
            nsample = min(args.cpu_sample, nrec)
            val, times, So, oo = cpu_reference(d, nsample, ncores, steps=1, keep=True)
            line["cpu_baseline"] = {"value": val, "unit": "records/s", "cores": ncores,
                                    "kind": "port",
                                    "sample": f"first {nsample} records, one sparse data loop"}
    ctx.close()
    if not args.profile and rank == 0:
        line["parity"] = bench_parity(mp, local, d, nsample, So, oo)
    if not args.profile:
        line["structure"] = structure_measure(mp, S, pinned, local, host_struct_s, ncores)
    if args.brokenlines > 0 and rank == 0 and not args.profile:
        line["brokenlines"] = brokenlines_measure(mp, local, args.brokenlines, ncores)
    if args.serve_jobs > 0 and rank == 0 and not args.profile:
        line["serving"] = serve_measure(mp, local, njobs=args.serve_jobs)
    if args.minres_iters > 0 and rank == 0 and not args.profile:
        line["minres"] = minres_measure(mp, local, iters=args.minres_iters, ncores=ncores)
        if args.whole_job:
            cpu_rate = line.get("cpu_baseline", {}).get("value")
            line["whole_job"] = whole_job_measure(mp, d, local, cpu_rate,
                                                  line["minres"]["cpu_baseline"]["ms_per_iteration"],
                                                  pinned=pinned)
    if args.dense_n > 0 and rank == 0 and not args.profile:
        line["dense_solve"] = dense_solve_measure(mp, local, nmod=args.dense_n // 10,
                                                  ntracks=20 * args.dense_n, sqminl=args.dense_sqminl,
                                                  cond=args.dense_cond, skip_slow=args.dense_n > 40000)
    for arr in pinned:
        arr.free()
    if rank == 0:
        print(json.dumps(line))
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()

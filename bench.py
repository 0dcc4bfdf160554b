#!/usr/bin/env python3
"""Steady-state HEOM solves/s on GB300: the serial double-quantum-dot model (nd = 16,
truncation tier 4: 30453 ADOs, 393812 stored entries) over a sweep of bias points,
solved by the mixed-precision batched TFQMR (FP32x2 arithmetic, FP64 refinement) to
||b - A x|| <= crit, with the plain FP64 GPU solve and the CPU restatement timed beside.

One step = one batched solve of B bias points from the Boltzmann initial guess.
`value` times device-resident solves; `e2e` times the same batch through the C ABI with
host buffers (initial guesses and parameters in, steady states out).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "heom-quick2_gb300"))

METRIC = "HEOM steady solves/s & matvec GB/s: mixed vs FP64 GPU at 1e-8 current err"
WORKLOAD = "serial double quantum dot nd=16, tier L=4 (30453 ADOs, 393812 stored entries), Pade M=3, T=0.1, W=10"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--batch", type=int, default=8, help="bias points per solve (per GPU)")
    ap.add_argument("--crit", type=float, default=1e-9)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the records of the other configurations (crit 1e-10, the 128-instance sweep, "
                         "the Kanamori batch, the gradients) that follow the headline")
    ap.add_argument("--profile", action="store_true",
                    help="profiler run: warm-up solves, then one timed mixed solve; prints one short line")
    ap.add_argument("--profile-inner", action="store_true",
                    help="profiler run of the two fused FP32x2 inner-iteration kernels: 3 warm-up + 2 timed launches each")
    ap.add_argument("--inner-layout", default=None,
                    help="--profile-inner, --profile: the instance layout GxL (interleave G, L instances per lane, "
                         "e.g. 8x2) instead of the one the batch solves use")
    ap.add_argument("--profile-cheb", action="store_true",
                    help="profiler run of the FP32x2 Chebyshev propagation of the headline model (V = 0.8): 2 "
                         "warm-up and 3 timed steps of 0.05 (one kernel per Chebyshev term)")
    ap.add_argument("--profile-apply", default=None, choices=["fp64", "fp32x2", "fp32"],
                    help="profiler run of the apply alone over the batch: 3 warm-up + 2 timed launches")
    ap.add_argument("--workload", default="steady", choices=["steady", "dos", "jacobi"],
                    help="steady: batched steady states (the headline); dos: spectral function over frequencies; "
                         "jacobi: steady state by the reference's Jacobi sweeps")
    ap.add_argument("--freqs", type=int, default=8, help="dos: frequencies per step")
    ap.add_argument("--profile-cf", action="store_true",
                    help="dos: profiler run of the correlation-function apply alone: 3 warm-up + 2 timed launches")
    ap.add_argument("--profile-jacobi", action="store_true",
                    help="jacobi: profiler run of the sweep kernels alone: 1 + 3 launches of each")
    return ap.parse_args()


def bias_points(n):
    """Bias sweep centred on V = 0.8 (meV): V_b uniformly spaced in [0.4, 1.2]."""
    return [0.8] if n == 1 else [0.4 + 0.8 * b / (n - 1) for b in range(n)]


def rank_bias_points(batch, rank, world_size):
    """Replicas (weak scaling): rank r solves its own batch of bias points out of one sweep of
    batch * world_size points, so every rank does the same amount of distinct work."""
    pts = bias_points(batch * world_size)
    return pts[rank * batch:(rank + 1) * batch]


def max_over_ranks(x, dist, device="cpu"):
    """The largest per-rank value (the job's time), through an all-reduce; x itself without dist."""
    if not dist:
        return x
    import torch

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if ws > 1:
        import torch.distributed as dist  # noqa: F811

        backend = "nccl" if args.impl == "gb300" else "gloo"
        if backend == "nccl":
            import torch

            torch.cuda.set_device(local)
        dist.init_process_group(backend=backend)
    return ws, rank, local, dist


def clocks_start():
    path = os.path.join(tempfile.gettempdir(), f"heom_clocks_{os.getpid()}.csv")
    q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    try:
        f = open(path, "w")
        p = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200"],
                             stdout=f, stderr=subprocess.DEVNULL)
        return p, f, path
    except (OSError, FileNotFoundError):
        return None, None, path


def clocks_stop(h, gpu):
    p, f, path = h
    if p is None:
        return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
    p.terminate()
    p.wait()
    f.close()
    sm, mx, reasons = [], None, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in open(path):
        parts = [x.strip() for x in line.split(",")]
        if len(parts) < 9 or parts[0] != str(gpu):
            continue
        try:
            sm.append(float(parts[1]))
            mx = float(parts[2])
        except ValueError:
            continue
        for k, name in enumerate(names):
            if parts[5 + k].lower() == "active":
                reasons.add(name)
    os.unlink(path)
    return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
            "samples": len(sm)}


def measured_peak_hbm():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profile_traffic(name, key="dram_bytes_per_launch"):
    """DRAM bytes per launch of a kernel from a committed ncu summary under profiles/, if any."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(path):
            if line.startswith(key + ":"):
                return float(line.split(":")[1].split()[0])
    except (OSError, ValueError):
        pass
    return None


def cpu_reference(cfgs, nthreads, crit):
    """The oracle (C restatement of the reference FP64 path) on the host cores: one solve."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_ffi

    m = oracle_ffi.Model(cfgs[0])
    t0 = time.perf_counter()
    rho, info = m.solve_tfqmr(crit=crit, maxit0=20000, nthreads=nthreads)
    dt = time.perf_counter() - t0
    return dt, m.current(rho)[0].sum(), info


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo), and its logical core count."""
    name = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                name = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    if not name:
        try:
            for line in open("/proc/cpuinfo"):
                if line.lower().startswith(("model name", "cpu part")):
                    name = line.split(":", 1)[1].strip()
                    break
        except OSError:
            pass
    return name or "unknown", os.cpu_count() or 1


def cpu_one_thread_sample(cfg, applies_per_solve, napply=3):
    """The oracle's apply on one host thread: napply applies timed, scaled to one solve by the
    applies the FP64 TFQMR takes (the vector updates of TFQMR are a few percent beside them)."""
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_ffi

    m = oracle_ffi.Model(cfg)
    rng = np.random.default_rng(1)
    x = rng.standard_normal(m.lunk + 1) + 1j * rng.standard_normal(m.lunk + 1)
    m.calc_ax(x, nthreads=1)
    t0 = time.perf_counter()
    for _ in range(napply):
        x = m.calc_ax(x * 1e-3, nthreads=1)
    t_apply = (time.perf_counter() - t0) / napply
    return t_apply, 1.0 / (t_apply * applies_per_solve)


def sweep_record(crit):
    """The batched I-V sweep: 128 single-orbital instances with uneven hierarchies (seed
    20261203: V ~ U[-1, 1], U in {1, 2, 3}, eps = -U/2, tier in {2, 3, 4}), one table family
    solved as one batch on the tier-4 tables with each instance truncated at its own tier
    (heomq.sweep); wall time includes the host set-up of the tables.  Errors against the same
    sweep refined in FP64 to ||b - A x|| <= 1e-12.  A leg that does not reach crit is recorded
    as it ends."""
    import numpy as np

    import heomq
    from heomq import sweep

    cfgs = heomq.models.iv_sweep(128, seed=20261203)
    out = {"instances": len(cfgs), "groups": len(sweep.group_instances(cfgs)), "crit": crit}
    ref, _ = sweep.solve_sweep(cfgs, crit=1e-12, precision=heomq.PREC_FP64_REFINED, max_refine=16)
    for key, prec in (("mixed", heomq.PREC_MIXED), ("fp64", heomq.PREC_FP64)):
        sweep.solve_sweep(cfgs, crit=crit, precision=prec, check=False)            # warm-up
        t0 = time.perf_counter()
        cur, infos = sweep.solve_sweep(cfgs, crit=crit, precision=prec, check=False)
        wall = time.perf_counter() - t0
        dev = sum(i.seconds for i in infos)
        out[key] = {"wall_s": wall, "device_s": dev, "solves_per_s": len(cfgs) / wall,
                    "worst_current_rel_err": float(np.max(np.abs(cur - ref) / np.abs(ref))),
                    "converged": all(bool(i.converged) for i in infos), "resid": max(i.resid for i in infos),
                    "applies": max(i.iters for i in infos)}
    return out


def kanamori_record(crit):
    """The three-orbital Kanamori impurity (nd = 64, tier 2, Pade M = 6, T = 0.05): four bias
    points in one batch, and the single point V = 0.2 at crit 1e-10 (sub-record "v_0.2").
    Mixed precision against the plain FP64 TFQMR (which sits at the edge of its floor on the
    batch: it converges or stalls near 4e-8 depending on the rounding of its apply, and is
    recorded as it ends), both against FP64 inner solves refined to 1e-12."""
    import numpy as np
    import torch

    import heomq

    m = heomq.Model(heomq.models.HUND_L2)
    ctx = heomq.Context(m, adjoint=False)
    hb = 0.658211928
    L = m.lunk

    def bias_batch(Vs):
        es = np.array([[V / 2, V / 2, -V / 2, -V / 2] for V in Vs]) / hb
        es = np.ascontiguousarray(es.reshape(len(Vs), 2, 2).transpose(0, 2, 1).reshape(len(Vs), 4))
        return heomq.Batch(ctx, eshift_batch=es, nbatch=len(Vs))

    def record(Vs, c):
        batch = bias_batch(Vs)
        x0 = torch.zeros((len(Vs), batch.stride), dtype=torch.complex128, device="cuda")
        x0[:, :L] = torch.from_numpy(m.initial_guess()).cuda()
        x = torch.empty_like(x0)

        def solve(prec, cc, refine=8):
            x.copy_(x0)
            torch.cuda.synchronize()
            info = batch.solve_dev(x.data_ptr(), crit=cc, precision=prec, max_refine=refine, check=False)
            return info, np.array([ctx.current(x[b, :L].cpu().numpy())[0].sum() for b in range(len(Vs))])

        iref, ref = solve(heomq.PREC_FP64_REFINED, 1e-12, 16)
        out = {"bias_points": [round(v, 4) for v in Vs], "crit": c, "reference_resid": iref.resid}
        for key, prec in (("mixed", heomq.PREC_MIXED), ("fp64", heomq.PREC_FP64)):
            info, cur = solve(prec, c)
            out[key] = {"device_s": info.seconds, "applies": info.iters, "converged": bool(info.converged),
                        "resid": info.resid, "worst_current_rel_err": float(np.max(np.abs(cur - ref) / np.abs(ref)))}
        out["speedup_mixed_vs_fp64"] = out["fp64"]["device_s"] / out["mixed"]["device_s"]
        batch.close()
        return out

    out = {"workload": "Kanamori 3-orbital nd=64, tier 2 (7477 ADOs, 464968 entries), M=6, T=0.05"}
    out.update(record([0.4 + 0.8 * b / 3 for b in range(4)], crit))
    # the configuration's own point, V = 0.2, at the criterion that brings its current error
    # below 1e-8 (at 1e-9 the current sits 4e-8 from the reference there)
    out["v_0.2"] = record([0.2], 1e-10)
    ctx.close()
    return out


def gradient_record():
    """Adjoint gradients on the headline model (double dot, tier 4, M = 3): the steady
    dI_L/d{V, Gamma, U, eps} by the adjoint solve, against central differences (h = 1e-4,
    steady states refined to 1e-12); and the gradient of int I_L dt over 1000 Chebyshev steps of
    0.05 from the V = 0 steady state under the step bias 0.8, with checkpoints every 32 steps,
    against central differences of two forward runs (h = 1e-5)."""
    import heomq

    hb = 0.658211928
    p0 = dict(V=0.8, gamma=0.5, U=2.0, eps=-1.0)

    def cfg(**over):
        p = dict(p0)
        p.update(over)
        return heomq.models.dqd(ntier=5, nmats=3, **p)

    def current(c):
        m = heomq.Model(c)
        ctx = heomq.Context(m, adjoint=False)
        rho, _ = ctx.solve_tfqmr(crit=1e-12, precision=heomq.PREC_FP64_REFINED, max_refine=16)
        return ctx.current(rho)[0].sum()

    m = heomq.Model(cfg())
    nd2 = m.nrho ** 2
    import numpy as np

    du, de = m.get("dhs_du", nd2, np.complex128), m.get("dhs_deps", nd2, np.complex128)
    ctx = heomq.Context(m, dhs=(du, de))
    rho, _ = ctx.solve_tfqmr(crit=1e-12, precision=heomq.PREC_FP64_REFINED, max_refine=16)
    deshift = np.array([[0.5, 0.5], [-0.5, -0.5]]).T.reshape(-1) / hb
    t0 = time.perf_counter()
    dI, ainfo = ctx.steady_gradient(rho, deshift=deshift, gamma=p0["gamma"], dhs_du=du, dhs_deps=de, which=0xF,
                                    crit=1e-12)
    t_adj = time.perf_counter() - t0
    t0 = time.perf_counter()
    dmx, minfo = ctx.steady_gradient(rho, deshift=deshift, gamma=p0["gamma"], dhs_du=du, dhs_deps=de, which=0xF,
                                     crit=1e-12, precision=heomq.PREC_MIXED)
    t_mx = time.perf_counter() - t0
    steady = {"adjoint_s": t_adj, "adjoint_applies": ainfo.iters, "dI": dict(zip(("V", "gamma", "U", "eps"), map(float, dI))),
              "mixed_adjoint": {"adjoint_s": t_mx, "applies": minfo.iters, "refinements": minfo.refinements,
                                "converged": bool(minfo.converged),
                                "max_rel_diff_vs_fp64": float(np.max(np.abs(dmx - dI)) / np.max(np.abs(dI)))}}
    rel = {}
    for k, key in enumerate(("V", "gamma", "U")):
        h = 1e-4 * max(1.0, abs(p0[key]))
        fd = (current(cfg(**{key: p0[key] + h})) - current(cfg(**{key: p0[key] - h}))) / (2 * h)
        rel[key] = abs(dI[k] - fd) / abs(fd)
    steady["rel_err_vs_central_differences"] = rel
    ctx.close()
    # time-dependent: from the V = 0 steady state, 1000 Chebyshev steps of 0.05 under the step bias
    m0 = heomq.Model(cfg(V=0.0))
    c0 = heomq.Context(m0, adjoint=False)
    rho_eq, _ = c0.solve_tfqmr(crit=1e-12, precision=heomq.PREC_FP64_REFINED, max_refine=16)
    c0.close()
    amps, tchar = m.field()
    ctx = heomq.Context(m)
    t0 = time.perf_counter()
    J, dJ = ctx.td_gradient(rho_eq, 0.05, 1000, checkpoint_every=32)
    t_grad = time.perf_counter() - t0
    t0 = time.perf_counter()
    Jm, dJm = ctx.td_gradient(rho_eq, 0.05, 1000, checkpoint_every=32, method=heomq.PROP_CHEBYSHEV_MIXED)
    t_grad_mx = time.perf_counter() - t0

    def integral(scale, method=heomq.PROP_CHEBYSHEV):
        c = heomq.Context(m, adjoint=False, amps=scale * amps, tchar=tchar)
        t = time.perf_counter()
        _, jt = c.propagate(rho_eq, 0.0, 0.05, 1000, method=method, currents=True)
        dt = time.perf_counter() - t
        c.close()
        return 0.05 * jt[:, 0::m.nalf].sum(), dt

    jp, t_fwd = integral(1 + 1e-5)
    jm, _ = integral(1 - 1e-5)
    fd = (jp - jm) / 2e-5
    j1, _ = integral(1.0)
    jmx, t_mx = integral(1.0, heomq.PROP_CHEBYSHEV_MIXED)
    ctx.close()
    td = {"steps": 1000, "dt": 0.05, "checkpoint_every": 32, "forward_s": t_fwd, "gradient_s": t_grad,
          "dJ_dA": dJ, "central_difference": fd, "rel_err": abs(dJ - fd) / abs(fd),
          "forward_mixed_s": t_mx, "integral_rel_diff_mixed_vs_fp64": abs(jmx / j1 - 1),
          "gradient_mixed_s": t_grad_mx, "dJ_dA_mixed_rel_diff_vs_fp64": abs(dJm / dJ - 1)}
    return {"model": "serial double dot nd=16, tier 4, M=3", "steady": steady, "chebyshev": td}


def run_reference(args, ws, rank, dist):
    import heomq.models as models

    if rank != 0:
        return 0
    nthreads = os.cpu_count() or 1
    cfgs = [models.dqd(ntier=5, nmats=3, V=v) for v in bias_points(args.batch)]
    for _ in range(args.warmup):
        cpu_reference(cfgs[:1], nthreads, args.crit)
    times = []
    for k in range(args.steps):
        dt, _, _ = cpu_reference([cfgs[k % len(cfgs)]], nthreads, args.crit)
        times.append(dt)
    total = sum(times)
    value = args.steps / total
    line = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": {"workload": WORKLOAD, "batch": 1, "crit": args.crit, "solver": "TFQMR FP64 (oracle restatement)"},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": nthreads, "kind": "port",
                         "cpu_model": cpu_model()[0],
                         "sample": "one full FP64 TFQMR solve of one bias point per step (OpenMP over ADOs)"},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_gb300(args, ws, rank, local, dist):
    import numpy as np
    import torch

    import heomq

    dev = local
    torch.cuda.set_device(dev)
    B = args.batch
    Vs = rank_bias_points(B, rank, ws)
    cfg = heomq.models.dqd(ntier=5, nmats=3, V=0.8)
    model = heomq.Model(cfg)
    ctx = heomq.Context(model, device=dev, adjoint=False)
    hb = 0.658211928
    es = np.zeros((B, 2, 2))
    for b, V in enumerate(Vs):   # eleadinfty(ialf, ispin) = +-V/2 / hbar, (nalf, nspin) column-major per instance
        es[b] = np.array([[V / 2, V / 2], [-V / 2, -V / 2]]) / hb
    es_cm = np.ascontiguousarray(np.transpose(es, (0, 2, 1)).reshape(B, 4))
    batch = heomq.Batch(ctx, eshift_batch=es_cm, nbatch=B)
    L = model.lunk
    stride = batch.stride
    x0h = model.initial_guess()
    x0 = torch.zeros((B, stride), dtype=torch.complex128, device="cuda")
    x0[:, :L] = torch.from_numpy(x0h).to("cuda")
    x = torch.empty_like(x0)

    def step(prec, crit=None, refine=8, check=True, interleave=0, lane_instances=0):
        x.copy_(x0)
        torch.cuda.synchronize()
        return batch.solve_dev(x.data_ptr(), crit=crit or args.crit, precision=prec, max_refine=refine, check=check,
                               interleave=interleave, lane_instances=lane_instances)

    if args.profile_cheb:
        pm = heomq.Model(heomq.models.dqd(ntier=5, nmats=3, V=0.8))
        pc = heomq.Context(pm, device=dev, adjoint=False)
        r0 = pm.initial_guess()
        pc.propagate(r0, 0.0, 0.05, 2, method=heomq.PROP_CHEBYSHEV_MIXED)
        t0 = time.perf_counter()
        pc.propagate(r0, 0.0, 0.05, 3, method=heomq.PROP_CHEBYSHEV_MIXED)
        print(json.dumps({"profile_cheb": True, "entries": pm.lunk, "steps": 3,
                          "ms_per_step": 1e3 * (time.perf_counter() - t0) / 3}), flush=True)
        pc.close()
        batch.close()
        ctx.close()
        return 0
    if args.profile_apply:
        prec = {"fp64": heomq.PREC_FP64, "fp32x2": heomq.PREC_MIXED, "fp32": heomq.PREC_MIXED_FP32}[args.profile_apply]
        sec, alg = ctx.bench_apply(prec, reps=2, nbatch=B)
        print(json.dumps({"profile_apply": args.profile_apply, "batch": B, "apply_us": sec * 1e6,
                          "alg_bytes": alg}), flush=True)
        batch.close()
        ctx.close()
        return 0
    if args.profile_inner:
        if args.inner_layout:
            g, lanes = (int(v) for v in args.inner_layout.split("x"))
            (sb, sa), (bb, ba) = ctx.bench_inner_layout(g, lanes, reps=2, nbatch=B)
        else:
            (sb, sa), (bb, ba) = ctx.bench_inner(heomq.PREC_MIXED, reps=2, nbatch=B)
        print(json.dumps({"profile_inner": True, "batch": B, "layout": args.inner_layout or "of the solves",
                          "k_in_b_us": sb * 1e6, "k_in_a_us": sa * 1e6, "alg_bytes": [bb, ba]}), flush=True)
        batch.close()
        ctx.close()
        return 0
    for _ in range(args.warmup):
        step(heomq.PREC_MIXED)
    # the automatic layout choice of the inner kernels times one solve with each candidate first
    while ctx.tuned_layout(B) == (0, 0):
        step(heomq.PREC_MIXED)
    layout = ctx.tuned_layout(B)
    if args.profile:
        # under a profiler the timed choice of the layout is distorted: --inner-layout names it
        g, lanes = (int(v) for v in args.inner_layout.split("x")) if args.inner_layout else (0, 0)
        info = step(heomq.PREC_MIXED, interleave=g, lane_instances=lanes)
        print(json.dumps({"profile_run": True, "batch": B, "applies": info.iters, "seconds": info.seconds,
                          "launches": info.launches}), flush=True)
        batch.close()
        ctx.close()
        return 0
    # the instance layouts the automatic choice compares: one solve and the two fused kernels each
    layouts = {}
    for g, lanes in heomq.layout_candidates(B):
        (kb, ka), _ = ctx.bench_inner_layout(g, lanes, reps=10, nbatch=B)
        layouts[f"{g}x{lanes}"] = {"solve_ms": 1e3 * step(heomq.PREC_MIXED, interleave=g, lane_instances=lanes).seconds,
                                   "k_in_b_us": kb * 1e6, "k_in_a_us": ka * 1e6}
    # FP64 GPU path beside (same batch, same criterion)
    info64 = step(heomq.PREC_FP64)
    cur64 = [ctx.current(x[b, :L].cpu().numpy())[0].sum() for b in range(B)]

    clk = clocks_start() if rank == 0 else None
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    dev_s, launches = 0.0, 0
    infos = []
    for _ in range(args.steps):
        info = step(heomq.PREC_MIXED)
        dev_s += info.seconds
        launches += info.launches
        infos.append(info)
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    if dist:
        dist.barrier()
    clocks = clocks_stop(clk, dev) if rank == 0 else None
    curm = [ctx.current(x[b, :L].cpu().numpy())[0].sum() for b in range(B)]
    t_step = max_over_ranks(dev_s / args.steps, dist, device="cuda")
    value = ws * B / t_step

    # FP64 timing beside (one step, after the timed region)
    t64 = info64.seconds
    # end to end through the C ABI with host buffers: every step copies the initial guesses
    # and the lead shifts in (the batch shares the context's H, which is not sent) and the
    # steady states out; the median over the same number of steps as the headline
    pinned = torch.empty((B, L), dtype=torch.complex128, pin_memory=True)
    rhos = pinned.numpy()
    e2e_times = []
    for _ in range(args.steps):
        rhos[:] = x0h
        t0 = time.perf_counter()
        out, info_e = ctx.solve_batch(rhos, eshift_batch=es_cm, crit=args.crit, precision=heomq.PREC_MIXED,
                                      inplace=True)
        jt = [ctx.current(out[b])[0].sum() for b in range(B)]
        e2e_times.append(time.perf_counter() - t0)
    e2e_value = ws * B / max_over_ranks(statistics.median(e2e_times), dist, device="cuda")
    h2d = rhos.nbytes + es_cm.nbytes
    d2h = rhos.nbytes

    # roofline of the dominant kernel: the first fused kernel of an inner TFQMR iteration
    # (apply of w + the first half of the vector updates) over the batch; the second one and
    # the plain apply beside it
    (sb, sa), (bb, ba) = ctx.bench_inner(heomq.PREC_MIXED, reps=20, nbatch=B)
    sec, alg_bytes = ctx.bench_apply(heomq.PREC_MIXED, reps=20, nbatch=B)
    sec64, alg64 = ctx.bench_apply(heomq.PREC_FP64, reps=10, nbatch=B)
    peak, peak_kind = measured_peak_hbm()
    achieved = bb / sb / 1e9
    # ncu summary of the fused kernels in the chosen layout
    prof = {(8, 1): "inner_fp32x2_interleaved_dqd_L4_batch8.md",
            (8, 2): "inner_fp32x2_interleaved_pairs_dqd_L4_batch8.md"}.get(layout, "inner_fp32x2_dqd_L4_batch8.md")
    traffic = profile_traffic(prof, "dram_bytes_per_launch_k_in_b")
    traffic_a = profile_traffic(prof, "dram_bytes_per_launch_k_in_a")
    # accuracy: both paths against a reference steady state refined in FP64 to ||b - A x|| <= 1e-12
    # (mixed refinement; FP64 TFQMR alone stalls near 2e-10 on this model)
    info_ref = step(heomq.PREC_FP64_REFINED, crit=1e-12, refine=16, check=False)
    curt = [ctx.current(x[b, :L].cpu().numpy())[0].sum() for b in range(B)]
    err = max(abs(a - b) / abs(b) for a, b in zip(curm, curt))
    err64 = max(abs(a - b) / abs(b) for a, b in zip(cur64, curt))

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        model_name, nthreads = cpu_model()
        cfg0 = heomq.models.dqd(ntier=5, nmats=3, V=Vs[0])
        dt, jcpu, cinfo = cpu_reference([cfg0], nthreads, args.crit)
        t1, v1 = cpu_one_thread_sample(cfg0, info64.iters)
        cpu = {"value": 1.0 / dt, "unit": "solves/s", "cores": nthreads, "kind": "port", "cpu_model": model_name,
               "sample": f"one FP64 TFQMR solve of one bias point (V={Vs[0]:.2f}) by the C oracle, OpenMP over ADOs",
               "current_rel_diff_vs_gpu_fp64": abs(jcpu - cur64[0]) / abs(cur64[0]),
               "one_thread": {"value": v1, "unit": "solves/s", "cores": 1, "apply_s": t1,
                              "sample": f"3 applies of the oracle on one thread, scaled by the {info64.iters} "
                                        "applies of the FP64 TFQMR solve"}}
    configs = None
    if rank == 0 and not args.no_configs:
        # the criterion of the mixed-versus-FP64 configuration (FP64 refinement to 1e-10)
        ts, c10 = [], None
        for _ in range(3):
            i10 = step(heomq.PREC_MIXED, crit=1e-10)
            ts.append(i10.seconds)
        c10 = [ctx.current(x[b, :L].cpu().numpy())[0].sum() for b in range(B)]
        configs = {
            "crit_1e-10": {"solves_per_s": B / statistics.median(ts), "applies_per_solve": i10.iters,
                           "resid": i10.resid, "current_rel_err": max(abs(a - b) / abs(b) for a, b in zip(c10, curt))},
            "iv_sweep_128": sweep_record(args.crit),
            "kanamori_nd64": kanamori_record(args.crit),
            "gradients_dqd_L4": gradient_record(),
        }

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32x2+f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "batch": B, "bias_points_meV": [round(v, 4) for v in Vs],
                       "crit": args.crit, "solver": "TFQMR in FP32x2 on the regularised operator, FP64 residual refinement",
                       "l2": f"inputs larger than L2: {B} x 9 solver vectors x {L * 16 / 1e6:.1f} MB",
                       "parallelism": f"replicas x{ws}", "wall_s": wall,
                       "applies_per_solve": infos[-1].iters, "refinements": infos[-1].refinements,
                       "inner_layout": {"chosen": f"{layout[0]}x{layout[1]}", "candidates": layouts,
                                        "key": "GxL: G instances interleaved per entry group, L per thread"},
                       "fp64": {"solves_per_s": ws * B / t64, "applies_per_solve": info64.iters,
                                "apply_us": sec64 * 1e6, "apply_gbs_alg": alg64 / sec64 / 1e9},
                       "speedup_mixed_vs_fp64": (ws * B / t_step) / (ws * B / t64),
                       "current_rel_err_mixed": err, "current_rel_err_fp64": err64,
                       "current_reference": "steady state refined with FP64 inner solves to ||b - A x|| <= 1e-12",
                       "current_reference_resid": info_ref.resid, "other_configurations": configs},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": f"k_in_b<FP32x2, regularised>, layout {layout[0]}x{layout[1]}: apply of w plus "
                                   "the fused vector updates, over the batch",
                         "kernel_us": sb * 1e6, "alg_bytes_per_launch": bb,
                         "k_in_a": {"kernel_us": sa * 1e6, "alg_bytes_per_launch": ba, "achieved": ba / sa / 1e9,
                                    "traffic": traffic_a},
                         "plain_apply": {"kernel_us": sec * 1e6, "alg_bytes_per_launch": alg_bytes,
                                         "achieved": alg_bytes / sec / 1e9},
                         "note": "the apply inside is issue-bound on the FP32/ALU pipes (double-float arithmetic); "
                                 "the fused vector updates use the HBM bandwidth it leaves idle: profiles/" + prof},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    batch.close()
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return 0


DOS_METRIC = "HEOM spectral-function frequencies/s (corrfunc frequency domain): mixed vs FP64 GPU"
DOS_WORKLOAD = ("spectral function A(w) of a_(1,up) of the serial double quantum dot nd=16, tier L=4 "
                "(correlation-function pattern: 670672 entries per component), steady state at V=0.8, "
                "two FP64 TFQMR solves per frequency to ||b - L x|| <= crit")
DOS_CRIT = 1e-8


def dos_freqs(n):
    import numpy as np

    return np.linspace(-3.0, 3.0, n)


def cpu_dos_sample(nthreads, applies_per_freq, napply=40):
    """The oracle's C restatement of calc_ax_cf_spa_omp on the host cores: `napply` applies
    timed, scaled to one frequency by the applies the same TFQMR takes per frequency."""
    import numpy as np

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_ffi
    import heomq.models as models

    m = oracle_ffi.Model(models.dqd(ntier=5, nmats=3, V=0.8))
    c = oracle_ffi.CF(m, 1, 1)
    rng = np.random.default_rng(1)
    xh = rng.standard_normal(c.lunkcf) + 1j * rng.standard_normal(c.lunkcf)
    xa = rng.standard_normal(c.lunkcf) + 1j * rng.standard_normal(c.lunkcf)
    c.apply(0.3, 1, xh, xa, nthreads=nthreads)
    t0 = time.perf_counter()
    for _ in range(napply):
        xh, xa = c.apply(0.3, 1, xh * 1e-3, xa * 1e-3, nthreads=nthreads)
    t_apply = (time.perf_counter() - t0) / napply
    return t_apply, 1.0 / (t_apply * applies_per_freq)


def run_dos_reference(args, ws, rank, dist):
    if rank != 0:
        return 0
    nthreads = os.cpu_count() or 1
    # applies per frequency of the FP64 TFQMR at this criterion (two solves of at most 750
    # applies each), the count the GPU path measured for the same algorithm on this workload
    applies = 2 * 750
    for _ in range(args.warmup):
        cpu_dos_sample(nthreads, applies, napply=2)
    vals, per = [], []
    for _ in range(args.steps):
        t_apply, v = cpu_dos_sample(nthreads, applies, napply=10)
        vals.append(v)
        per.append(t_apply)
    value = statistics.median(vals)
    line = {
        "metric": DOS_METRIC, "value": value, "unit": "freqs/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 / value, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": {"workload": DOS_WORKLOAD, "crit": DOS_CRIT, "apply_s": statistics.median(per),
                   "applies_per_frequency": applies},
        "cpu_baseline": {"value": value, "unit": "freqs/s", "cores": nthreads, "kind": "port",
                         "sample": "10 applies of the C restatement of calc_ax_cf_spa_omp (OpenMP over ADOs) per step, "
                                   f"scaled by {applies} applies per frequency"},
        "e2e": {"value": value, "unit": "freqs/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_dos(args, ws, rank, local, dist):
    import numpy as np
    import torch

    import heomq

    dev = local
    torch.cuda.set_device(dev)
    model = heomq.Model(heomq.models.dqd(ntier=5, nmats=3, V=0.8))
    ctx = heomq.Context(model, device=dev, adjoint=False)
    cf = heomq.CorrFunc(ctx, 1, 1)
    nf = args.freqs
    freqs = dos_freqs(nf * ws)[rank * nf:(rank + 1) * nf]
    if args.profile_cf:
        sec, alg = cf.bench_apply(nbatch=2 * nf, reps=2)
        (sb, sa), _ = cf.bench_inner(nbatch=2 * nf, reps=2)
        print(json.dumps({"profile_cf": True, "instances": 2 * nf, "apply_us": sec * 1e6, "alg_bytes": alg,
                          "k_in_b_us": sb * 1e6, "k_in_a_us": sa * 1e6}), flush=True)
        return 0
    rho, sinfo = ctx.solve_tfqmr(crit=1e-10, precision=heomq.PREC_MIXED)
    mixed = heomq.PREC_MIXED
    for _ in range(args.warmup):
        cf.dos(rho, freqs, crit=DOS_CRIT, precision=mixed)
    clk = clocks_start() if rank == 0 else None
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    dev_s, wall_s, launches, infos = 0.0, [], 0, []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        out, info = cf.dos(rho, freqs, crit=DOS_CRIT, precision=mixed)
        wall_s.append(time.perf_counter() - t0)
        dev_s += info.seconds
        launches += info.launches
        infos.append(info)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = clocks_stop(clk, dev) if rank == 0 else None
    t_step = max_over_ranks(dev_s / args.steps, dist, device="cuda")
    value = ws * nf / t_step
    e2e_value = ws * nf / max_over_ranks(statistics.median(wall_s), dist, device="cuda")
    # the FP64 reference algorithm beside (one step, after the timed region)
    out64, info64 = cf.dos(rho, freqs, crit=DOS_CRIT)
    dos_err = float(np.max(np.abs(out[:, 0] - out64[:, 0]) / np.abs(out64[:, 0])))
    sec, alg = cf.bench_apply(nbatch=2 * nf, reps=10)
    (sb, sa), (bb, ba) = cf.bench_inner(nbatch=2 * nf, reps=10)
    peak, peak_kind = measured_peak_hbm()
    achieved = bb / sb / 1e9
    prof = "inner_cf_fp32x2_pairs_dqd_L4_16inst.md"
    traffic = profile_traffic(prof, "dram_bytes_per_launch_k_in_b")
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        nthreads = os.cpu_count() or 1
        applies = 2 * info64.iters
        t_apply, v = cpu_dos_sample(nthreads, applies, napply=20)
        cpu = {"value": v, "unit": "freqs/s", "cores": nthreads, "kind": "port",
               "sample": f"20 applies of the C restatement of calc_ax_cf_spa_omp (OpenMP over ADOs, {t_apply * 1e3:.1f} ms "
                         f"each), scaled by the {applies} applies per frequency the same FP64 TFQMR took on the GPU "
                         "(batch maximum per solve)"}
    if rank == 0:
        n = model.nrho
        line = {
            "metric": DOS_METRIC, "value": value, "unit": "freqs/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32x2+f64", "data": "synthetic",
            "config": {"workload": DOS_WORKLOAD, "freqs_per_step": nf, "freq_range_eV": [-3.0, 3.0], "crit": DOS_CRIT,
                       "solver": "FP32x2 fused inner TFQMR, FP64 residual refinement",
                       "fp64": {"freqs_per_s": ws * nf / info64.seconds, "applies_per_solve_max": info64.iters,
                                "resid_max": info64.resid},
                       "speedup_mixed_vs_fp64": info64.seconds / t_step, "dos_rel_diff_mixed_vs_fp64": dos_err,
                       "solves_per_step": 2 * nf, "applies_per_solve_max": infos[-1].iters,
                       "resid_max": infos[-1].resid, "converged": bool(infos[-1].converged),
                       "l2": f"inputs larger than L2: {2 * nf} instances x 12 vectors x {2 * cf.lunkcf * 16 / 1e6:.1f} MB",
                       "parallelism": f"frequencies split over {ws} replicas",
                       "spectrum_min": float(out[:, 1:3].min()), "steady_resid": sinfo.resid},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "peak_kind": peak_kind,
                         "kernel": f"k_in_b<FP32x2, cf>, two instances per lane: apply of w plus the fused vector updates, "
                                   f"over {2 * nf} instances",
                         "kernel_us": sb * 1e6, "alg_bytes_per_launch": bb,
                         "k_in_a": {"kernel_us": sa * 1e6, "alg_bytes_per_launch": ba, "achieved": ba / sa / 1e9},
                         "fp64_apply": {"kernel_us": sec * 1e6, "alg_bytes_per_launch": alg, "achieved": alg / sec / 1e9,
                                        "profile": "profiles/apply_cf_fp64_dqd_L4_16inst.md"},
                         "note": "issue-bound on the FP32/ALU pipes like the steady inner kernels: profiles/" + prof},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "freqs/s", "h2d_bytes_per_step": model.lunk * 16 + nf * 8,
                    "d2h_bytes_per_step": nf * 5 * 8},
            "gpu_launches": launches,
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    cf.close()
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return 0


JAC_METRIC = "HEOM Jacobi steady solves/s (methodss = 4, FP64)"
JAC_WORKLOAD = ("steady state of the serial double quantum dot nd=16, tier L=4 (393812 stored entries), V=0.8, "
                "by Jacobi sweeps with prelude_jacobi's shift to ||A x - e_trace|| <= crit")
JAC_CRIT = 1e-9


def cpu_jacobi_sample(nthreads, sweeps, nsample=2):
    """The oracle's C restatement of calc_ax_jacobi_spa_omp (Liouville-space eigenvectors,
    OpenMP over ADOs): `nsample` sweeps timed, scaled to a solve of `sweeps` sweeps."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_ffi
    import heomq.models as models

    os.environ.setdefault("OMP_NUM_THREADS", str(nthreads))
    m = oracle_ffi.Model(models.dqd(ntier=5, nmats=3, V=0.8))
    J = oracle_ffi.Jacobi(m)
    x = m.initial_guess()
    x = J.sweep(x)
    t0 = time.perf_counter()
    for _ in range(nsample):
        x = J.sweep(x)
    t_sweep = (time.perf_counter() - t0) / nsample
    return t_sweep, 1.0 / (t_sweep * sweeps)


def run_jacobi_reference(args, ws, rank, dist):
    if rank != 0:
        return 0
    nthreads = os.cpu_count() or 1
    sweeps = 451   # the sweeps the same iteration takes on this workload (measured on the GPU path)
    cpu_jacobi_sample(nthreads, sweeps, nsample=1)
    vals, per = [], []
    for _ in range(args.steps):
        t_sweep, v = cpu_jacobi_sample(nthreads, sweeps, nsample=1)
        vals.append(v)
        per.append(t_sweep)
    value = statistics.median(vals)
    line = {
        "metric": JAC_METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 / value, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
        "config": {"workload": JAC_WORKLOAD, "crit": JAC_CRIT, "sweep_s": statistics.median(per), "sweeps": sweeps},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": nthreads, "kind": "port",
                         "sample": f"one sweep of the C restatement of calc_ax_jacobi_spa_omp per step, scaled by {sweeps} sweeps"},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_jacobi(args, ws, rank, local, dist):
    import torch

    import heomq

    dev = local
    torch.cuda.set_device(dev)
    model = heomq.Model(heomq.models.dqd(ntier=5, nmats=3, V=0.8))
    ctx = heomq.Context(model, device=dev, adjoint=False)
    if args.profile_jacobi:
        t_jac, t_app, b, f = ctx.bench_jacobi(reps=3)
        print(json.dumps({"profile_jacobi": True, "transform_us": t_jac * 1e6, "apply_us": t_app * 1e6}), flush=True)
        return 0
    x0 = model.initial_guess()
    for _ in range(args.warmup):
        ctx.solve_jacobi(x0, crit=JAC_CRIT, maxit0=20000)
    clk = clocks_start() if rank == 0 else None
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    dev_s, wall, launches, infos = 0.0, [], 0, []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        rho, info = ctx.solve_jacobi(x0, crit=JAC_CRIT, maxit0=20000)
        wall.append(time.perf_counter() - t0)
        dev_s += info.seconds
        launches += info.launches
        infos.append(info)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clocks = clocks_stop(clk, dev) if rank == 0 else None
    t_step = max_over_ranks(dev_s / args.steps, dist, device="cuda")
    value = ws / t_step
    e2e_value = ws / max_over_ranks(statistics.median(wall), dist, device="cuda")
    t_jac, t_app, jbytes, jcfma = ctx.bench_jacobi(reps=10)
    ref, _ = ctx.solve_tfqmr(crit=1e-10, precision=heomq.PREC_MIXED)
    cur_err = abs(ctx.current(rho)[0].sum() / ctx.current(ref)[0].sum() - 1)
    peak, peak_kind = measured_peak_hbm()
    achieved = jbytes / t_jac / 1e9
    prof = "jacobi_sweep_dqd_L4.md"
    cpu = None
    sweeps = infos[-1].iters + 1
    if rank == 0 and not args.no_cpu_baseline:
        nthreads = os.cpu_count() or 1
        t_sweep, v = cpu_jacobi_sample(nthreads, sweeps)
        cpu = {"value": v, "unit": "solves/s", "cores": nthreads, "kind": "port",
               "sample": f"2 sweeps of the C restatement of calc_ax_jacobi_spa_omp (Liouville-space eigenvectors, "
                         f"OpenMP over ADOs, {t_sweep:.2f} s each), scaled by the {sweeps} sweeps of the solve"}
    if rank == 0:
        line = {
            "metric": JAC_METRIC, "value": value, "unit": "solves/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": JAC_WORKLOAD, "crit": JAC_CRIT, "ejac_eV": ctx.jacobi_shift() * 0.658211928,
                       "sweeps": sweeps, "resid": infos[-1].resid, "converged": bool(infos[-1].converged),
                       "current_rel_diff_vs_mixed_tfqmr": cur_err,
                       "l2": f"inputs larger than L2: 3 vectors x {model.lunk * 16 / 1e6:.1f} MB plus the plan",
                       "parallelism": f"replicas x{ws}", "apply_us": t_app * 1e6},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": profile_traffic(prof), "peak_kind": peak_kind,
                         "kernel": "k_jacobi: per-ADO sector transform of one sweep", "kernel_us": t_jac * 1e6,
                         "alg_bytes_per_launch": jbytes, "complex_fma_per_launch": jcfma,
                         "fp64_tflops": 8 * jcfma / t_jac / 1e12,
                         "note": "FP64 small dense products per ADO from shared memory; profiles/" + prof},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": "solves/s", "h2d_bytes_per_step": model.lunk * 16,
                    "d2h_bytes_per_step": model.lunk * 16},
            "gpu_launches": launches,
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    ctx.close()
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    ws, rank, local, dist = dist_setup(args)
    if args.impl == "reference":
        if args.workload == "dos":
            return run_dos_reference(args, ws, rank, dist)
        if args.workload == "jacobi":
            return run_jacobi_reference(args, ws, rank, dist)
        return run_reference(args, ws, rank, dist)
    sys.path.insert(0, ROOT)
    import __graft_entry__

    if rank == 0:
        __graft_entry__.build()
    if dist:
        dist.barrier()
    if args.workload == "dos":
        return run_dos(args, ws, rank, local, dist)
    if args.workload == "jacobi":
        return run_jacobi(args, ws, rank, local, dist)
    return run_gb300(args, ws, rank, local, dist)


if __name__ == "__main__":
    sys.exit(main())

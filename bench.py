"""Benchmark of the Davidson sigma path (sigma = H.C and S^2.C) on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--n-det N]

Workload: 14 alpha + 14 beta electrons in 80 MOs (N_int = 2), 1e6 seeded
determinants (aufbau reference + random <=4-fold excitations), seeded integrals
(h_pp ~ U[-2,2] sorted, h_pq ~ N(0,0.02), (pq|rs) = sum_k L^k_pq L^k_rs with 120
factors L ~ N(0,0.05)), 4 states.  One step is one sigma application on all
N_det rows for the 4 states.  The determinant set's connectivity and matrix
elements are built once (qpgpu_set_dets, the provider rebuild after TOUCH
psi_det) outside the timed region and reported as `setup_s`; Davidson calls
sigma ~10-30 times per determinant set.

value      FP64 sigma on device-resident vectors (kernel path), det*state/s
e2e        FP64 sigma through qpgpu_h_s2_u0 with host (pinned) buffers,
           host<->device copies inside the timed region
sigma_fp32 FP32 matrix elements x FP32 coefficients with Kahan sums
roofline   dominant kernel k_sigma64: algorithmic bytes per launch
           B = N*N_st*8*3 + N*(2*N_int*8+12) + P*N_st*8 over its CUDA-event time
cpu_baseline  the CPU oracle (C++ restatement of H_S2_u_0_nstates_openmp,
           OpenMP dynamic,64, all host threads): one full sigma of all N_det rows
           in bilinear order for the 4 states (the converged Davidson vectors when
           the Davidson block runs; its output gives the oracle energies)
davidson   time-to-E of each arm against the oracle's FP64 energies: the
           Rayleigh quotients of the oracle's sigma on the converged vectors
--impl reference: that CPU path alone, as the reference arm, each step a
           contiguous block of bilinear rows (the blocks of all steps tile the set).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

METRIC = "Davidson time-to-E (≤1e-6 Ha vs FP64) & σ det·states/s: mixed+learned vs plain"
UNIT = "det*state/s"
N_STATES = 4


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n-det", type=int, default=1_000_000)
    ap.add_argument("--reference-budget-s", type=float, default=150.0,
                    help="wall-time budget of the whole --impl reference run (warm-up + timed steps)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-davidson", action="store_true", help="skip the Davidson time-to-E block")
    ap.add_argument("--davidson-only", action="store_true", help="only the Davidson block (profiling)")
    ap.add_argument("--batch", action="store_true",
                    help="add the batched block: 64 independent CI problems solved together vs one by one")
    ap.add_argument("--batch-only", action="store_true", help="only the batched block")
    ap.add_argument("--c1", action="store_true",
                    help="only the 1e4-determinant, 40-MO Davidson: device vs the oracle's CPU Davidson")
    ap.add_argument("--n-states-diag", type=int, default=8, help="N_st_diag of the Davidson runs")
    ap.add_argument("--davidson-sze-max", type=int, default=10, help="davidson_sze_max of the Davidson runs")
    return ap.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
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
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = float(f[1])
            except ValueError:
                continue
            for nm, v in zip(names, f[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profiled_traffic(N, P):
    """dram bytes per k_sigma64 launch from the committed ncu summary, scaled to this workload."""
    p = os.path.join(ROOT, "profiles", "sigma_fp64_ncu.json")
    if not os.path.exists(p):
        return None, None
    with open(p) as f:
        d = json.load(f)
    try:
        scale = P / float(d["n_pairs"])
        return float(d["dram_bytes_per_launch"]) * scale, d.get("note")
    except (KeyError, ZeroDivisionError):
        return None, None


def cpu_model():
    """CPU model name of this host (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except (OSError, subprocess.SubprocessError):
        pass
    try:
        with open("/proc/cpuinfo") as f:
            for ln in f:
                if ln.lower().startswith("model name"):
                    return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


def oracle_full_sigma(prob, u):
    """The CPU oracle's sigma on all N_det rows of u (N_st, N) in psi_det order:
    returns (v, s, seconds, threads, oracle).  The determinant index (the
    providers) is built before the clock starts, as the GPU set-up is."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle, num_threads
    o = Oracle.from_problem(prob)
    t = time.perf_counter()
    v, s = o.h_s2_u0(u)
    dt = time.perf_counter() - t
    return v, s, dt, num_threads(), o


def cpu_baseline_entry(n_det, nst, seconds, threads, what):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import build_flags
    return {"value": n_det * nst / seconds, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"all {n_det} rows (contiguous, bilinear order), {nst} states, one full sigma of {what}: "
                      f"{seconds:.1f} s",
            "flags": build_flags(), "cpu_model": cpu_model()}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from quantum_package_gb300 import generate as G
    prob = G.make_problem(2, n_det=args.n_det, n_states=N_STATES)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle, build_flags, num_threads
    o = Oracle.from_problem(prob)
    u_t = np.ascontiguousarray(G.random_coefficients(prob.n_det, N_STATES, prob.seed).T)
    N = prob.n_det
    # each step is one contiguous block of bilinear rows (so the reference's
    # kcol_prev reuse of the beta-singles scan works as in a full sigma); the
    # blocks of the warm-up and timed steps start at evenly spaced rows and
    # together tile the set, their size bounded so the run fits the budget
    nblk = max(1, args.steps + args.warmup)
    t = time.perf_counter()
    mid = N // 2
    o.h_s2_u0_work(u_t, mid + 1, min(N, mid + 2000), 0, 1)
    rows_per_s = min(2000, N - mid) / max(time.perf_counter() - t, 1e-6)
    per_step_s = args.reference_budget_s / nblk
    span = (N + nblk - 1) // nblk
    B = int(max(1, min(span, rows_per_s * per_step_s)))
    starts = [1 + i * span for i in range(nblk)]
    for i in range(args.warmup):
        o.h_s2_u0_work(u_t, starts[i], min(N, starts[i] + B - 1), 0, 1)
    rows = 0
    t = time.perf_counter()
    for i in range(args.warmup, nblk):
        iend = min(N, starts[i] + B - 1)
        o.h_s2_u0_work(u_t, starts[i], iend, 0, 1)
        rows += max(0, iend - starts[i] + 1)
    dt = time.perf_counter() - t
    val = rows * N_STATES / dt
    sample = (f"contiguous blocks of {B} bilinear rows starting every {span} rows of {N} "
              f"({rows} rows over {args.steps} steps, {N_STATES} states)")
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(prob),
        "cpu_baseline": {"value": val, "unit": UNIT, "cores": num_threads(), "kind": "port", "sample": sample,
                         "flags": build_flags(), "cpu_model": cpu_model()},
        "e2e": {"value": val, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU oracle (C++ FP64 restatement of u0Hu0.irp.f:97-448, OpenMP dynamic,64); the Fortran "
                "reference cannot be compiled here (no gfortran/irpf90)",
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_config(prob):
    return {"workload": "sigma H.C+S2.C, 14a+14b in 80 MOs (N_int=2), 1e6 seeded dets, 4 states",
            "n_det": prob.n_det, "n_mo": prob.n_mo, "n_alpha": prob.n_alpha, "n_beta": prob.n_beta,
            "n_states": N_STATES, "seed": prob.seed,
            "l2": "inputs larger than L2 (stored pairs ~12 GB FP64 per sigma)"}


N_STATES_DIAG = 8
SZE_MAX = 8
E_TOL = 1e-6


def _guess(n, seed):
    """Unit vector on the reference determinant + seeded Gaussian extra vectors."""
    rng = np.random.default_rng(seed)
    u = rng.normal(size=(N_STATES_DIAG, n))
    u[0] = 0.0
    u[0, 0] = 1.0
    return u


def _time_to_e(res, e_ref, fp64):
    """ms from the Davidson call until an FP64 (or float-float) sigma iteration has every state within
    E_TOL of e_ref; FP32-sigma iterations do not count."""
    tr = res["trace"]
    de = np.abs(tr["energies"] - e_ref[None, :]).max(axis=1)
    ok = np.where((de < E_TOL) & (tr["precision"] != 1))[0]  # FP64 or float-float iterations (not FP32)
    return (float(tr["elapsed_ms"][ok[0]]) if len(ok) else None), int(ok[0] + 1) if len(ok) else None


def davidson_block(prob, wf):
    """Time-to-E of the 4 lowest states: plain FP64 Davidson vs mixed precision vs
    mixed precision + learned preconditioner (trained on the first 1e4 and 2e5
    determinants of the same draw, as earlier CIPSI stages).  Returns the
    block's settings, the raw runs and the tight FP64 run whose eigenvectors the
    oracle checks; davidson_finish turns the runs into times against the
    oracle's energies."""
    from quantum_package_gb300 import ALGEBRA_FP64, ALGEBRA_TC, FF, FP32
    N = prob.n_det
    u = _guess(N, prob.seed)
    kw = dict(n_states=N_STATES, s2_eig=False, max_iter=400, davidson_sze_max=SZE_MAX)
    tight = wf.davidson_diag_hs2(u, threshold=1e-12, **kw)
    # one-time costs of the FP32 path (module load, launch-shape tuning for this
    # determinant set) outside the timed runs, as the set-up is
    wf.davidson_diag_hs2(u, threshold=1e-10, precision=FP32, **dict(kw, max_iter=3))
    out = {"n_states": N_STATES, "n_states_diag": N_STATES_DIAG, "davidson_sze_max": SZE_MAX,
           "threshold": 1e-10, "e_tol_ha": E_TOL,
           "note": "s2_eig off: the seeded space is not spin complete; energies are electronic (Ha)"}
    raw = {}

    def run(name, **extra):
        raw[name] = wf.davidson_diag_hs2(u, threshold=1e-10, **kw, **extra)

    run("plain_fp64")
    run("mixed", precision=FP32)
    # the specification's split: FP32 sigma with the FP64 sigma at each restart,
    # projections, Gram-Schmidt, Ritz vectors, step and residual norms in FP64
    run("mixed_spec", precision=FP32, algebra=ALGEBRA_FP64)
    # the same split with the FP64-accurate Gram blocks on the tensor cores
    run("mixed_spec_tc", precision=FP32, algebra=ALGEBRA_TC)
    # restart (defect-correction) sigma in float-float instead of FP64
    run("mixed_ff_restart", precision=FF)
    # learned preconditioner: earlier stages of the same determinant draw
    t0 = time.perf_counter()
    wf.mlp_init(seed=3)
    train = {}
    for n_stage in (10_000, 200_000):
        if n_stage >= N:
            continue
        wf.set_dets(prob.dets[:n_stage])
        r = wf.davidson_diag_hs2(_guess(n_stage, prob.seed), threshold=1e-10, collect_every=1, collect_max=16,
                                 preconditioner=1 if train else 0, **kw)
        loss = wf.mlp_train(epochs=20, batch=4096, lr=2e-3, seed=4)
        train[str(n_stage)] = {"n_sigma": r["n_sigma"], "samples": int(r["n_samples"]), "loss": loss}
    wf.set_dets(prob.dets)
    wf.davidson_diag_hs2(u, threshold=1e-10, precision=FP32, **dict(kw, max_iter=3))  # tuning, as above
    out["training"] = {"stages": train, "wall_s": time.perf_counter() - t0,
                       "note": "training on earlier determinant sets; not part of time-to-E"}
    # learned step in place of the diagonal step (preconditioner=1), and as an
    # extra direction in the slots of the non-target Ritz vectors (=2)
    run("plain_fp64_learned", preconditioner=1)
    run("mixed_learned", precision=FP32, preconditioner=1)
    run("mixed_learned_extra", precision=FP32, preconditioner=2)
    run("mixed_ff_restart_learned_extra", precision=FF, preconditioner=2)
    return out, raw, tight


def oracle_energies(prob, vecs, v, s, o):
    """Rayleigh quotients of the oracle's sigma on the vectors vecs (N_st, N),
    with the residual norms |Hu - Eu| / |u| and the reference's convergence
    measure (the squared norm of the Davidson step, diagonalization_hs2.irp.f:386-395)."""
    hjj, _ = o.diag()
    sz = 0.5 * (prob.n_alpha - prob.n_beta)
    sz2sz = sz * (sz - 1.0)
    uu = np.einsum("ij,ij->i", vecs, vecs)
    e = np.einsum("ij,ij->i", vecs, v) / uu
    s2 = np.einsum("ij,ij->i", vecs, s) / uu + sz2sz
    r = v - e[:, None] * vecs
    res = np.sqrt(np.einsum("ij,ij->i", r, r) / uu)
    step = (-r) * (1.0 + s2[:, None] * vecs - s - sz2sz) / np.maximum(hjj[None, :] - e[:, None], 1e-2)
    return e, res, np.einsum("ij,ij->i", step, step)


def davidson_finish(out, raw, e_ref):
    from quantum_package_gb300 import FP64
    for name, r in raw.items():
        t, it = _time_to_e(r, e_ref, FP64)
        out[name] = {"time_to_E_s": t / 1e3 if t is not None else None, "iterations_to_E": it,
                     "n_sigma": r["n_sigma"], "converged": r["converged"],
                     "total_s": float(r["trace"]["elapsed_ms"][-1]) / 1e3,
                     "max_dE_ha": float(np.abs(r["energies"][:N_STATES] - e_ref).max()),
                     "n_fallback": r["n_fallback"]}
    for arm in raw:
        if arm == "plain_fp64":
            continue
        a, b = out["plain_fp64"]["time_to_E_s"], out[arm]["time_to_E_s"]
        out[f"speedup_{arm}_vs_plain"] = (a / b) if (a and b) else None
    return out


def c1_block(nsd=4, sze_max=10, threshold=1e-10):
    """10 alpha + 10 beta electrons in 40 MOs (N_int = 1), 1e4 seeded determinants, 1 state:
    the device Davidson (FP64, mixed) against the oracle's CPU Davidson (the C++ restatement of
    davidson_diag_hjj_sjj over the OpenMP sigma, all host threads), same guess and threshold.
    The device runs report time-to-E (first FP64 iteration within 1e-6 Ha of the converged
    energy) and total time; the CPU run reports its total time to the threshold."""
    from quantum_package_gb300 import FP32, FP64
    from quantum_package_gb300 import generate as G
    from quantum_package_gb300.sigma import Wavefunction
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from oracle import Oracle
    prob = G.make_problem(1)
    N = prob.n_det
    rng = np.random.default_rng(prob.seed)
    u = rng.normal(size=(nsd, N))
    u[0] = 0.0
    u[0, 0] = 1.0
    o = Oracle.from_problem(prob)
    t = time.perf_counter()
    eo, _, _, n_sigma_cpu, res_cpu = o.davidson(u, 1, davidson_sze_max=sze_max, threshold=threshold, s2_eig=False,
                                                 max_sigma=1000)
    cpu_s = time.perf_counter() - t
    wf = Wavefunction.from_problem(prob)
    kw = dict(n_states=1, s2_eig=False, max_iter=1000, davidson_sze_max=sze_max)
    e_ref = np.asarray(eo[:1])
    out = {"workload": "Davidson, 10a+10b in 40 MOs (N_int=1), 1e4 seeded dets, 1 state",
           "n_states_diag": nsd, "davidson_sze_max": sze_max, "threshold": threshold,
           "cpu_oracle": {"total_s": cpu_s, "n_sigma": int(n_sigma_cpu), "energy": float(eo[0]),
                          "threads": os.cpu_count()}}
    for name, prec in (("device_fp64", FP64), ("device_mixed", FP32)):
        wf.davidson_diag_hs2(u, threshold=threshold, precision=prec, **kw)  # warm-up (module load, tuning)
        r = wf.davidson_diag_hs2(u, threshold=threshold, precision=prec, **kw)
        t_e, it = _time_to_e(r, e_ref, FP64)
        out[name] = {"time_to_E_s": t_e / 1e3 if t_e is not None else None, "iterations_to_E": it,
                     "total_s": float(r["trace"]["elapsed_ms"][-1]) / 1e3, "n_sigma": r["n_sigma"],
                     "converged": r["converged"], "dE_vs_cpu_ha": float(abs(r["energies"][0] - eo[0]))}
    return out


def batch_block(n_problems=64):
    """64 independent CI problems (30-60 MOs, 8-16 electrons per spin, N_det
    log-uniform 1e3-1e5, 1-3 states, seeded): the batched Davidson (one
    persistent sigma launch per iteration for all problems, graph replay,
    autotuned shape) against the same problems solved one after the other,
    FP64, threshold 1e-10, N_st_diag = 4."""
    import torch
    from quantum_package_gb300 import FP64
    from quantum_package_gb300 import generate as G
    from quantum_package_gb300.batch import Batch
    from quantum_package_gb300.sigma import Wavefunction
    t0 = time.perf_counter()
    probs = G.batched_problems(n_problems)
    gen_s = time.perf_counter() - t0
    wfs = [Wavefunction.from_problem(p) for p in probs]
    setup_s = sum(w.info()["setup_ms"] for w in wfs) / 1e3
    nsd = 4
    guesses = []
    for i, p in enumerate(probs):
        rng = np.random.default_rng(p.seed)
        g = rng.normal(size=(nsd, p.n_det))
        g[0] = 0.0
        g[0, 0] = 1.0
        guesses.append(g)
    nst = [p.n_states for p in probs]
    b = Batch(wfs)
    b.davidson(guesses, nst, threshold=1e-10, precision=FP64, max_iter=400)  # autotune + graph capture
    torch.cuda.synchronize()
    t = time.perf_counter()
    r = b.davidson(guesses, nst, threshold=1e-10, precision=FP64, max_iter=400)
    torch.cuda.synchronize()
    batched_s = time.perf_counter() - t
    for w, g, k in zip(wfs, guesses, nst):  # warm each problem's own path once
        w.davidson_diag_hs2(g, n_states=k, threshold=1e-10, s2_eig=False, max_iter=3)
    torch.cuda.synchronize()
    t = time.perf_counter()
    single = [w.davidson_diag_hs2(g, n_states=k, threshold=1e-10, s2_eig=False, max_iter=400)
              for w, g, k in zip(wfs, guesses, nst)]
    torch.cuda.synchronize()
    seq_s = time.perf_counter() - t
    de = max(float(np.abs(r["energies"][i, :k] - single[i]["energies"][:k]).max()) for i, k in enumerate(nst))
    b.close()
    st = r["stats"]
    return {"n_problems": n_problems, "total_dets": int(sum(p.n_det for p in probs)),
            "det_range": [int(min(p.n_det for p in probs)), int(max(p.n_det for p in probs))],
            "batched_s": batched_s, "sequential_s": seq_s, "speedup": seq_s / batched_s,
            "n_converged": int(st["n_converged"]), "n_iter": int(st["n_iter"]),
            "tuned_warps": int(st["tuned_warps"]), "tuned_blocks_per_sm": int(st["tuned_blocks_per_sm"]),
            "max_dE_batched_vs_single_ha": de, "setup_s_total": setup_s, "generate_s": gen_s,
            "note": "wall time of the Davidson calls (host loop included); set-up of the 64 determinant sets excluded"}


def run_ours(args):
    global N_STATES_DIAG, SZE_MAX
    N_STATES_DIAG = args.n_states_diag
    SZE_MAX = args.davidson_sze_max
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    from quantum_package_gb300 import FP32, FP64
    from quantum_package_gb300 import _lib
    from quantum_package_gb300 import generate as G
    from quantum_package_gb300.sigma import Wavefunction, stream_handle

    if args.batch_only:
        if rank == 0:
            print(json.dumps({"batch": batch_block()}), flush=True)
        return 0
    if args.c1:
        if rank == 0:
            print(json.dumps({"c1": c1_block()}), flush=True)
        return 0
    prob = G.make_problem(2, n_det=args.n_det, n_states=N_STATES)
    N = prob.n_det
    wf = Wavefunction.from_problem(prob)
    info = wf.info()
    P = info["n_pairs"]
    if args.davidson_only:
        d, raw, tight = davidson_block(prob, wf)
        d = davidson_finish(d, raw, tight["energies"][:N_STATES])
        d["e_ref"] = "the tight (1e-12) FP64 device run (--davidson-only skips the oracle)"
        if rank == 0:
            print(json.dumps({"davidson": d, "setup_s": info["setup_ms"] / 1e3}), flush=True)
        return 0
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    order = torch.from_numpy(wf.bilinear_order().astype(np.int64)).to(dev)
    u0 = torch.from_numpy(G.random_coefficients(N, N_STATES, prob.seed)).to(dev)
    ut = u0[:, order].T.contiguous()
    ut32 = ut.float()
    v = torch.empty_like(ut)
    s = torch.empty_like(ut)
    launches_per_sigma = 1 + (1 if info["n_split_rows"] > 0 else 0)

    def timed(prec, steps, warm):
        with torch.cuda.stream(stream):
            for _ in range(warm):
                wf.sigma_bilinear(v, s, ut, ut32, prec, stream)
            stream.synchronize()
            if world > 1:
                torch.distributed.barrier()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                wf.sigma_bilinear(v, s, ut, ut32, prec, stream)
            e1.record(stream)
            stream.synchronize()
        return e0.elapsed_time(e1) / steps

    with ClockSampler(local) as clk:
        ms64 = timed(FP64, args.steps, args.warmup)
    ms32 = timed(FP32, args.steps, args.warmup)
    if world > 1:
        t = torch.tensor([ms64], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms64 = float(t.item())

    # end to end through the C-ABI with host buffers (pinned)
    hu = torch.from_numpy(G.random_coefficients(N, N_STATES, prob.seed)).pin_memory()
    hv = torch.empty_like(hu).pin_memory()
    hs = torch.empty_like(hu).pin_memory()
    L = _lib.load()
    import ctypes as C

    def e2e_once():
        _lib.check(L.qpgpu_h_s2_u0(wf.ctx, C.c_void_p(hv.data_ptr()), C.c_void_p(hs.data_ptr()),
                                   C.c_void_p(hu.data_ptr()), N_STATES, N), wf.ctx)

    for _ in range(args.warmup):
        e2e_once()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_once()
    e2e_s = (time.perf_counter() - t0) / args.steps

    # correctness spot check of the e2e result against the device path
    ref = torch.empty_like(u0)
    refs = torch.empty_like(u0)
    wf.h_s2_u0_device(ref, refs, u0, FP64, torch.cuda.current_stream())
    torch.cuda.synchronize()
    rel = float((ref.cpu() - hv).abs().max() / ref.abs().max())

    peak, peak_kind = measured_peak_hbm()
    nint = prob.n_int
    alg_bytes = N * N_STATES * 8 * 3 + N * (2 * nint * 8 + 12) + P * N_STATES * 8
    stored_bytes = P * (4 + 8) + N * N_STATES * 8 * 3 + N * 28
    achieved = alg_bytes / (ms64 * 1e-3) / 1e9
    traffic, tnote = profiled_traffic(N, P)
    fp64_pipe = None
    try:
        with open(os.path.join(ROOT, "profiles", "sigma_fp64_ncu.json")) as f:
            fp64_pipe = json.load(f).get("fp64_pipe_active")
    except (OSError, ValueError):
        pass
    value = world * N * N_STATES / (ms64 * 1e-3)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms64, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(prob),
        "setup_s": info["setup_ms"] / 1e3,
        "n_pairs": P,
        "sigma_including_setup": N * N_STATES / (info["setup_ms"] * 1e-3 + ms64 * 1e-3),
        "sigma_fp32": {"value": N * N_STATES / (ms32 * 1e-3), "unit": UNIT, "ms_per_step": ms32,
                       "dtype": "f32 (Kahan sums, FP64 diagonal)"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                     "kernel": "k_sigma64<4>",
                     "fp64_pipe_active": fp64_pipe,
                     "bound_note": "the HBM fraction is reported as the contract asks; ncu shows the FP64 pipe "
                                   "(about 2 FMA/clk/SM on GB300) as the limiting unit (fp64_pipe_active)",
                     "algorithmic_bytes_per_launch": alg_bytes,
                     "stored_pair_bytes_per_launch": stored_bytes,
                     "stored_pair_frac": stored_bytes / (ms64 * 1e-3) / 1e9 / peak,
                     "note": "algorithmic bytes count one gather of C_J per pair (L2-resident at this size); "
                             "stored_pair_frac is the HBM fraction of the bytes the kernel must stream"},
        "e2e": {"value": N * N_STATES / e2e_s, "unit": UNIT, "h2d_bytes_per_step": N * N_STATES * 8,
                "d2h_bytes_per_step": 2 * N * N_STATES * 8, "max_rel_diff_vs_device": rel},
        "gpu_launches": launches_per_sigma * args.steps,
        "clocks": clk.summary(),
    }
    dav = raw = tight = None
    if not args.no_davidson:
        dav, raw, tight = davidson_block(prob, wf)
    if args.batch:
        line["batch"] = batch_block()
    # CPU leg after all GPU timing (rank 0): one full oracle sigma of the four
    # converged FP64 eigenvectors; its time is the CPU baseline, its Rayleigh
    # quotients the FP64 oracle energies every arm's time-to-E is judged against
    if rank == 0 and not args.no_cpu_baseline:
        vecs = tight["vectors"][:N_STATES] if tight is not None else G.random_coefficients(N, N_STATES, prob.seed)
        ov, os_, sec, thr, o = oracle_full_sigma(prob, vecs)
        line["cpu_baseline"] = cpu_baseline_entry(
            N, N_STATES, sec, thr, "the converged Davidson vectors" if tight is not None else "seeded vectors")
        if dav is not None:
            e_or, res_or, step_or = oracle_energies(prob, vecs, ov, os_, o)
            dav = davidson_finish(dav, raw, e_or)
            dav["oracle_energies"] = e_or.tolist()
            dav["oracle_residual_norms"] = res_or.tolist()
            dav["oracle_step_norms2"] = step_or.tolist()
            dav["gpu_tight_minus_oracle_ha"] = (tight["energies"][:N_STATES] - e_or).tolist()
            dav["e_ref"] = ("oracle: Rayleigh quotients of the CPU oracle's FP64 sigma on the eigenvectors of a "
                            "1e-12-converged FP64 device run")
        del o
    if dav is not None and "e_ref" not in dav:
        dav = davidson_finish(dav, raw, tight["energies"][:N_STATES])
        dav["e_ref"] = "the tight (1e-12) FP64 device run (CPU leg skipped)"
    if dav is not None:
        line["davidson"] = dav
    if traffic is not None:
        line["roofline"]["traffic_note"] = tnote
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())

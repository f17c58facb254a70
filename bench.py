"""Benchmark: direct-SCF Fock builds (J and K) per second on one GB300.

Workload (N=1): the (H2O)8 water cluster in the 6-31G-shaped basis
(104 Cartesian functions), Schwarz threshold 1e-12 -- a full J+K build per
step, every unique shell quartet computed once.  Synthetic, seeded geometry
(rchem_gb300.geometry.config("h2o8_631g")); the density is the core-guess
density of that system.

Timing: W warm-up builds, then K timed builds, each bracketed by CUDA events
that the library records on the stream its kernels run on (from the copy of D
in to the copies of J and K out, so host submission latency is excluded); a
256 MiB buffer is written between timed builds (outside the events) so L2
(~126 MB) holds nothing of the previous build.  ``value`` is FP64 Fock builds/s with D, J and K resident on the device;
``e2e`` is the same through the C ABI with host arrays (H2D of D and D2H of J
and K inside the timed region).  The mixed FP32/FP64 form is reported under
``forms``.

CPU baselines (rank 0, N=1): ``cpu_baseline`` is the reference's algorithm
on a bounded sample, as below; ``cpu_baseline_strong`` is a whole build by a
strong CPU code over the same integrals (8-fold symmetry, Schwarz screen,
OpenMP), with a one-core figure from a strided sample of the bra pairs.

--impl reference: the reference's algorithm (src/basis.rs:383-428 loops over
the THO integrals of libpyquante2/cints.c with its own Boys function), run by
the CPU oracle with all host threads on a bounded sample of J/K elements and
extrapolated to a whole build.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "h2o8_631g"
WORKLOAD_DESC = "(H2O)8 water cluster, 6-31G-shaped basis (104 Cartesian functions), direct-SCF J+K Fock build"
METRIC = "Fock builds/s"
NOMINAL_FP64_TFLOPS = 1.25


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=WORKLOAD)
    ap.add_argument("--cpu-sample", type=int, default=0, help="J/K elements timed for the CPU baseline (0: auto)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-targets", action="store_true",
                    help="skip the (H2O)32, 512-geometry batch and gradient measurements")
    return ap.parse_args()


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def core_guess_density(rc, b, nocc):
    S = rc.S(b)
    H = rc.T(b) + rc.V(b)
    w, U = np.linalg.eigh(S)
    X = U @ np.diag(w ** -0.5) @ U.T
    _, Cp = np.linalg.eigh(X.T @ H @ X)
    C = X @ Cp
    return C[:, :nocc] @ C[:, :nocc].T, H


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (FileNotFoundError, OSError):
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.lines:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def cpu_reference_rate(workload, sample, steps=1, boys_shipped=True, target_s=10.0):
    """The reference's JK_direct loops (2 THO ERIs per primitive quartet) on a
    seeded sample of J/K elements, all host threads; returns builds/s
    extrapolated to the n^2 elements of a build, threads and sample size.
    ``sample`` = 0 sizes the sample from a one-element-per-thread pilot so
    that each step takes about ``target_s`` seconds."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    import rchem_gb300 as rc

    bname, Z, R = rc.geometry.config(workload)
    ob = O.expand_basis(Z, R, rc.load_bse(bname))
    port = O.port()
    port.set_boys(not boys_shipped)
    threads = port.num_threads()
    n = ob.n
    rng = np.random.default_rng(17)
    X = rng.normal(size=(n, n))
    D = X @ X.T / n
    m = sample
    if not m:
        pm, pn = rng.integers(0, n, threads), rng.integers(0, n, threads)
        t0 = time.perf_counter()
        O.JK_direct_elements(ob, D, pm, pn)
        per_round = max(time.perf_counter() - t0, 1e-6)  # one element on every thread
        m = threads * int(min(max(1, round(target_s / per_round)), 4096))
    rates = []
    for s in range(steps):
        mus = rng.integers(0, n, m)
        nus = rng.integers(0, n, m)
        t0 = time.perf_counter()
        O.JK_direct_elements(ob, D, mus, nus)
        dt = time.perf_counter() - t0
        rates.append(m / (dt * n * n))
    port.set_boys(True)
    return rates, threads, m, n


def cpu_strong_rate(workload, D, J_ref=None, K_ref=None, tau=1e-12, target_1core_s=4.0):
    """A strong CPU Fock build with the reference's own integrals (THO ERIs,
    the shipped Boys function): each unique contracted integral once (8-fold
    symmetry), quartets with Q_ij Q_kl < tau skipped like the GPU build,
    OpenMP over all host threads.  All cores: one whole build timed.  One core:
    a strided subset of the bra pairs timed and extrapolated by the number of
    integrals that pass the screen."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    import rchem_gb300 as rc

    bname, Z, R = rc.geometry.config(workload)
    ob = O.expand_basis(Z, R, rc.load_bse(bname))
    port = O.port()
    port.set_boys(False)
    try:
        threads = port.num_threads()
        n = ob.n
        npair = n * (n + 1) // 2
        t0 = time.perf_counter()
        Q = O.schwarz(ob)
        t_q = time.perf_counter() - t0
        total = O.JK_sym_screened(ob, D, Q, tau, count_only=True)[2]
        t0 = time.perf_counter()
        J, K, cnt = O.JK_sym_screened(ob, D, Q, tau)
        t_all = time.perf_counter() - t0
        # one core: a pilot over every 97th bra pair sizes a strided sample of about target_1core_s
        pilot = np.arange(0, npair, 97)
        t0 = time.perf_counter()
        c_p = O.JK_sym_screened(ob, D, Q, tau, pairs=pilot, nthreads=1)[2]
        per_int = (time.perf_counter() - t0) / max(c_p, 1)
        stride = int(min(max(1, round(total * per_int / target_1core_s)), npair))
        sample = np.arange(stride // 2, npair, stride)
        t0 = time.perf_counter()
        c_1 = O.JK_sym_screened(ob, D, Q, tau, pairs=sample, nthreads=1)[2]
        t_1 = time.perf_counter() - t0
    finally:
        port.set_boys(True)
    out = {"value": 1.0 / t_all, "unit": "builds/s", "cores": threads, "kind": "port",
           "algorithm": "each unique contracted integral once (8-fold symmetry), Schwarz screen Q_ij Q_kl >= %g "
                        "over contracted functions, THO ERIs of libpyquante2/cints.c with the shipped Boys "
                        "function, OpenMP dynamic over bra pairs" % tau,
           "sample": "one whole build on all %d threads (%d contracted integrals)" % (threads, cnt),
           "schwarz_s": t_q,
           "one_core": {"value": c_1 / (t_1 * total), "unit": "builds/s", "cores": 1,
                        "sample": "%d of %d bra pairs (every %d-th), %d integrals, extrapolated to the %d of a "
                                  "build" % (len(sample), npair, stride, c_1, total)}}
    if J_ref is not None:
        out["max_abs_dJ_vs_gpu_fp64"] = float(np.abs(J - J_ref).max())
        out["max_abs_dK_vs_gpu_fp64"] = float(np.abs(K - K_ref).max())
    return out


def _timed_builds(rc, torch, b, D, tau32, reps=3, emulated=False):
    s = torch.cuda.Stream()
    b.set_stream(s.cuda_stream)
    J, K = torch.empty_like(D), torch.empty_like(D)
    for _ in range(2):
        rc.JK_direct(J, K, b, D, fp32_tau=tau32, emulated=emulated)
    ms = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(s)
        rc.JK_direct(J, K, b, D, fp32_tau=tau32, emulated=emulated)
        e1.record(s)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    return float(np.median(ms)), b.stats()


def hbm_context(traffic, ms):
    """DRAM bytes per build (ncu) against the measured copy bandwidth: shows the
    Fock build is not memory-bound."""
    try:
        peak = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))["hbm_gbs"]
    except (OSError, ValueError, KeyError):
        return None
    if not traffic:
        return {"peak_gbs": peak}
    gbs = traffic / (ms * 1e-3) / 1e9
    return {"achieved_gbs": gbs, "peak_gbs": peak, "frac": gbs / peak, "peak_source": "MEASURED_PEAKS.json"}


def target_workloads(rc, torch):
    """The targets stated on the larger workloads: mixed vs FP64 Fock build on
    (H2O)32 in the 6-31G*-shaped basis (608 functions) at converged-SCF
    |dE| <= 1 uEh, and the adjoint gradient time per geometry on (H2O)4 in the
    6-31G**-shaped basis (100 functions)."""
    out = {}
    bname, Z, R = rc.geometry.config("h2o32_631gs")
    with rc.Basis(Z, R, bname) as b:
        rc.scf.rhf(b, max_iter=2)  # warm-up: work plan, graph, cuSOLVER initialisation
        tuned = b.autotune(1e-12, 0.0)  # tile shapes per class list (and the large classes' kernel) for this form
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r64 = rc.scf.rhf(b, thresh_e=1e-10)
        t_scf64 = time.perf_counter() - t0
        D = r64["D"].contiguous()
        ms64, st64 = _timed_builds(rc, torch, b, D, 0.0)
        rec = {"nbf": b.nbf, "fp64_ms": ms64, "fp64_builds_per_s": 1000.0 / ms64, "eris_fp64": st64["eris_fp64"],
               "fp64_flops": st64["flops_fp64"], "scf_fp64_s": t_scf64, "scf_iterations": r64["iterations"],
               "e_total_fp64": r64["e_total"], "mixed": {},
               "warp_cooperative_lists_fp64": sorted(k for (k, p), v in tuned.items() if p == 0 and v == 0)}
        for tau32 in (1e-6, 1e-4):
            b.autotune(1e-12, tau32)
            ms, st = _timed_builds(rc, torch, b, D, tau32)
            t0 = time.perf_counter()
            r = rc.scf.rhf(b, thresh_e=1e-10, fp32_tau=tau32)
            t_scf = time.perf_counter() - t0
            rec["mixed"]["%g" % tau32] = {
                "ms": ms, "builds_per_s": 1000.0 / ms, "speedup_vs_fp64": ms64 / ms,
                "fp32_quartet_fraction": st["quartets_fp32"] / max(1, st["quartets_fp32"] + st["quartets_fp64"]),
                "scf_dE_Eh": r["e_total"] - r64["e_total"], "scf_max_dD": float((r["D"] - r64["D"]).abs().max()),
                "scf_s": t_scf, "scf_iterations": r["iterations"]}
        # emulated FP64 (double-float on the FP32 pipe), alone and under the mixed form
        rec["emulated"] = {}
        for tau32 in (0.0, 1e-6):
            b.autotune(1e-12, tau32, emulated=True)
            ms, st = _timed_builds(rc, torch, b, D, tau32, emulated=True)
            r = rc.scf.rhf(b, thresh_e=1e-10, fp32_tau=tau32, emulated=True)
            rec["emulated"]["fp32_tau=%g" % tau32] = {
                "ms": ms, "builds_per_s": 1000.0 / ms, "speedup_vs_fp64": ms64 / ms,
                "scf_dE_Eh": r["e_total"] - r64["e_total"], "scf_max_dD": float((r["D"] - r64["D"]).abs().max()),
                "scf_iterations": r["iterations"]}
        out["h2o32_631gs_fock"] = rec
    # 512 geometries of uneven size (monomer/dimer/trimer, 13/26/39 functions)
    # in one handle: every Fock build is one graph launch over all of them
    geoms = rc.geometry.water_batch(512, seed=7)
    bb = rc.batch.BatchBasis(geoms, "6-31g-fit")
    rc.batch.rhf_native(bb, max_iter=2)  # warm-up (plans, graphs)
    rc.batch.rhf_batch(bb, max_iter=2)
    rec = {"geometries": bb.ngeom, "packed_elements": bb.packed, "sizes": sorted(set(bb.geom_nbf.tolist())),
           "scf_driver": "rchem_rhf (the whole SCF loop in the library)"}
    for tag, tau32, emul in (("fp64", 0.0, False), ("mixed", 1e-6, False), ("emulated_mixed", 1e-6, True)):
        bb.autotune(1e-12, tau32, emulated=emul)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = rc.batch.rhf_native(bb, thresh_e=1e-10, fp32_tau=tau32, emulated=emul)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        g = rc.batch.gradient_batch(bb, r, fp32_tau=tau32, emulated=emul)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        rp = rc.batch.rhf_batch(bb, thresh_e=1e-10, fp32_tau=tau32, emulated=emul)
        torch.cuda.synchronize()
        t3 = time.perf_counter()
        rec[tag] = {"scf_s": t1 - t0, "gradient_s": t2 - t1, "s_per_geometry": (t2 - t0) / bb.ngeom,
                    "iterations": r["iterations"], "converged": r["converged"], "e_total": r["e_total"],
                    "python_driver_scf_s": t3 - t2,
                    "python_driver_max_abs_dE_Eh": float(np.abs(rp["e_total"] - r["e_total"]).max())}
    D = torch.zeros(bb.packed, dtype=torch.float64, device="cuda")
    J, K = torch.empty_like(D), torch.empty_like(D)
    rc.batch.jk(bb, D, J, K)
    for tag, tau32, emul in (("fp64", 0.0, False), ("mixed", 1e-6, False), ("emulated_mixed", 1e-6, True)):
        bb.autotune(1e-12, tau32, emulated=emul)
        rc.batch.jk(bb, D, J, K, fp32_tau=tau32, emulated=emul)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(3):
            rc.batch.jk(bb, D, J, K, fp32_tau=tau32, emulated=emul)
        torch.cuda.synchronize()
        rec[tag]["fock_build_all_geometries_ms"] = (time.perf_counter() - t0) / 3 * 1e3
    e64 = np.asarray(rec["fp64"].pop("e_total"))
    rec["mixed_vs_fp64_max_abs_dE_Eh"] = float(np.abs(np.asarray(rec["mixed"].pop("e_total")) - e64).max())
    rec["emulated_mixed_vs_fp64_max_abs_dE_Eh"] = float(
        np.abs(np.asarray(rec["emulated_mixed"].pop("e_total")) - e64).max())
    out["batch512_631g"] = rec
    bb.close()

    bname, Z, R = rc.geometry.config("h2o4_631gss")
    with rc.Basis(Z, R, bname) as b:
        rc.scf.gradient(b, rc.scf.rhf(b))  # warm-up (plans, graphs)
        b.autotune(1e-12, 0.0)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = rc.scf.rhf(b, thresh_e=1e-10)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        g = rc.scf.gradient(b, res)
        torch.cuda.synchronize()
        t2 = time.perf_counter()
        rec = {"nbf": b.nbf, "scf_s": t1 - t0, "gradient_s": t2 - t1, "s_per_geometry": t2 - t0,
               "max_abs_grad": float(g.abs().max()),
               "check": "central finite differences to 1e-6 Eh/bohr in tests/test_gpu_gradient.py"}
        # the same energy + gradient in the mixed and emulated+mixed forms
        for tag, tau32, emul in (("mixed", 1e-6, False), ("emulated_mixed", 1e-6, True)):
            b.autotune(1e-12, tau32, emulated=emul)
            rc.scf.gradient(b, rc.scf.rhf(b, fp32_tau=tau32, emulated=emul), fp32_tau=tau32, emulated=emul)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r2 = rc.scf.rhf(b, thresh_e=1e-10, fp32_tau=tau32, emulated=emul)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            g2 = rc.scf.gradient(b, r2, fp32_tau=tau32, emulated=emul)
            torch.cuda.synchronize()
            t2 = time.perf_counter()
            rec[tag] = {"scf_s": t1 - t0, "gradient_s": t2 - t1, "s_per_geometry": t2 - t0,
                        "dE_vs_fp64_Eh": r2["e_total"] - res["e_total"],
                        "max_abs_dgrad_vs_fp64": float((g2 - g).abs().max())}
        out["h2o4_631gss_gradient"] = rec
    return out


def run_reference(a):
    rank, world, _ = _dist()
    if rank != 0:
        return 0
    steps = max(1, a.steps)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    O.build_port()
    # each step about 8 s of CPU work, the whole run (steps + one warm-up) within about 2.5 minutes
    target = min(8.0, 150.0 / (steps + 1))
    cpu_reference_rate(a.workload, a.cpu_sample or 0, steps=1, target_s=0.2 * target)  # warm-up
    rates, threads, m, n = cpu_reference_rate(a.workload, a.cpu_sample, steps=steps, target_s=target)
    value = float(np.mean(rates))
    sample = ("%d J/K elements per step (seeded random (mu,nu)) of the %d x %d Fock matrix by the JK_direct loops "
              "(src/basis.rs:392-425), THO ERIs with the Numerical-Recipes Boys function as shipped; "
              "extrapolated to a full build" % (m, n, n))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "builds/s", "n_gpus": a.gpus,
        "steps": steps, "warmup": a.warmup, "ms_per_step": 1000.0 / value, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": a.workload, "description": WORKLOAD_DESC, "nbf": n},
        "cpu_baseline": {"value": value, "unit": "builds/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "builds/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main():
    a = _args()
    if a.impl == "reference":
        return run_reference(a)
    import torch

    rank, world, local = _dist()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    import rchem_gb300 as rc
    from rchem_gb300 import _lib

    bname, Z, R = rc.geometry.config(a.workload)
    nocc = int(sum(Z)) // 2
    b = rc.Basis(Z, R, bname)
    n = b.nbf
    stream = torch.cuda.Stream()
    b.set_stream(stream.cuda_stream)
    Dh, H = core_guess_density(rc, b, nocc)
    tuned = {"fp64": b.autotune(1e-12, 0.0)}  # per-class tile shapes for this basis (one-time set-up)
    D = torch.from_numpy(Dh).cuda()
    J = torch.empty_like(D)
    K = torch.empty_like(D)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def run(tau32, steps, warmup, emulated=False):
        # device time of each build from the library's own CUDA events on the
        # stream its kernels run on (bracketing the copy of D in, the class
        # kernels and the copies of J and K out); the L2 flush runs before.
        for _ in range(warmup):
            rc.JK_direct(J, K, b, D, fp32_tau=tau32, emulated=emulated)
        ms = []
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(1)
            rc.JK_direct(J, K, b, D, fp32_tau=tau32, emulated=emulated)
            ms.append(b.stats()["gpu_ms"])
        torch.cuda.synchronize()
        return ms

    # ---- timed region: FP64 form -----------------------------------------
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        ms64 = run(0.0, a.steps, a.warmup)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    st64 = b.stats()
    J64, K64 = J.cpu().numpy(), K.cpu().numpy()
    ms = float(np.mean(ms64))
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * 1000.0 / ms

    # ---- mixed form (same timing) -----------------------------------------
    tuned["mixed"] = b.autotune(1e-12, 1e-6)
    ms32 = run(1e-6, a.steps, a.warmup)
    st32 = b.stats()
    Jm, Km = J.cpu().numpy(), K.cpu().numpy()
    dE = float(np.sum(Dh * (2 * (Jm - J64) - (Km - K64))))  # energy change at fixed D, sum (H+F) o D
    ms_mixed = float(np.mean(ms32))

    # ---- emulated FP64 form (double-float on the FP32 pipe, same timing) ----
    tuned["emulated"] = b.autotune(1e-12, 0.0, emulated=True)
    msem = run(0.0, a.steps, a.warmup, emulated=True)
    stem = b.stats()
    Je, Ke = J.cpu().numpy(), K.cpu().numpy()
    ms_emul = float(np.mean(msem))
    # ---- emulated FP64 above fp32_tau = 1e-6, FP32 below ------------------
    tuned["emulated_mixed"] = b.autotune(1e-12, 1e-6, emulated=True)
    msem32 = run(1e-6, a.steps, a.warmup, emulated=True)
    Jem, Kem = J.cpu().numpy(), K.cpu().numpy()
    ms_emul32 = float(np.mean(msem32))

    # ---- end to end through the C ABI with host arrays ---------------------
    # D in, J and K out through pinned host buffers (numpy views of pinned
    # torch tensors): the library copies them on its own stream inside the call
    b.autotune(1e-12, 0.0)
    Dp = torch.from_numpy(Dh).pin_memory()
    Jp = torch.empty((n, n), dtype=torch.float64).pin_memory()
    Kp = torch.empty((n, n), dtype=torch.float64).pin_memory()
    Dpn, Jh, Kh = Dp.numpy(), Jp.numpy(), Kp.numpy()
    for _ in range(a.warmup):
        rc.JK_direct(Jh, Kh, b, Dpn)
    te = []
    for _ in range(a.steps):
        with torch.cuda.stream(stream):
            flush.fill_(1)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        rc.JK_direct(Jh, Kh, b, Dpn)
        te.append(time.perf_counter() - t1)
    e2e = world / float(np.mean(te))

    # ---- roofline: FP64 CUDA-core FMA pipe ---------------------------------
    import ctypes

    pk = ctypes.c_double(0.0)
    peak64 = None
    if _lib.lib().rchem_peak_fma(64, ctypes.byref(pk)) == 0:
        peak64 = pk.value
    pk32 = ctypes.c_double(0.0)
    peak32 = pk32.value if _lib.lib().rchem_peak_fma(32, ctypes.byref(pk32)) == 0 else None
    achieved = st64["flops_fp64"] / (ms * 1e-3) / 1e12
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tpath):
        try:
            traffic = json.load(open(tpath)).get(a.workload)  # bytes per build, all class kernels
        except (ValueError, OSError):
            traffic = None

    # ---- CPU baseline (rank 0, N=1 only) ------------------------------------
    cpu, cpu_strong = None, None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        rates, threads, m, _ = cpu_reference_rate(a.workload, a.cpu_sample, steps=1)
        cpu = {"value": rates[0], "unit": "builds/s", "cores": threads, "kind": "port",
               "sample": "%d J/K elements by the JK_direct loops (src/basis.rs:392-425) with THO ERIs and the "
                         "shipped NR Boys function, extrapolated to the %d^2 elements of a build" % (m, n)}
        cpu_strong = cpu_strong_rate(a.workload, Dh, J64, K64)

    # ---- the larger target workloads (outside the headline timed region) ------
    targets = None
    if rank == 0 and not a.no_targets:
        targets = target_workloads(rc, torch)

    clocks = clk.summary()
    launches = st64["kernels"] + 1  # class kernels + symmetrise
    line = {
        "metric": METRIC, "value": value, "unit": "builds/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic",
        "config": {"workload": a.workload, "description": WORKLOAD_DESC, "basis": bname, "nbf": n,
                   "schwarz_tau": 1e-12, "density": "core guess",
                   "tile_shapes": "rchem_autotune per class list before timing (min primitive quartets per lane)",
                   "l2": "256 MiB buffer written between timed steps (outside the events)"},
        "eris_per_s": st64["eris_fp64"] / (ms * 1e-3),
        "forms": {
            "fp64": {"builds_per_s": 1000.0 / ms, "ms": ms, "quartets": st64["quartets_fp64"],
                     "eris": st64["eris_fp64"], "prim_quartets": st64["prim_quartets_fp64"]},
            "mixed": {"builds_per_s": 1000.0 / ms_mixed, "ms": ms_mixed, "fp32_tau": 1e-6,
                      "quartets_fp64": st32["quartets_fp64"], "quartets_fp32": st32["quartets_fp32"],
                      "speedup_vs_fp64": ms / ms_mixed, "dE_fixed_density_Eh": dE,
                      "max_abs_dJ": float(np.abs(Jm - J64).max()), "max_abs_dK": float(np.abs(Km - K64).max())},
            "emulated": {"builds_per_s": 1000.0 / ms_emul, "ms": ms_emul, "speedup_vs_fp64": ms / ms_emul,
                         "arithmetic": "double-float (hi+lo float pairs) for classes up to total L 4, FP64 above",
                         "quartets": stem["quartets_fp64"],
                         "dE_fixed_density_Eh": float(np.sum(Dh * (2 * (Je - J64) - (Ke - K64)))),
                         "max_abs_dJ": float(np.abs(Je - J64).max()), "max_abs_dK": float(np.abs(Ke - K64).max())},
            "emulated_mixed": {"builds_per_s": 1000.0 / ms_emul32, "ms": ms_emul32, "fp32_tau": 1e-6,
                               "speedup_vs_fp64": ms / ms_emul32,
                               "dE_fixed_density_Eh": float(np.sum(Dh * (2 * (Jem - J64) - (Kem - K64)))),
                               "max_abs_dJ": float(np.abs(Jem - J64).max()),
                               "max_abs_dK": float(np.abs(Kem - K64).max())},
        },
        "e2e": {"value": e2e, "unit": "builds/s", "h2d_bytes_per_step": n * n * 8, "d2h_bytes_per_step": 2 * n * n * 8},
        "roofline": {"bound": "fp64", "achieved": achieved, "peak": peak64, "unit": "TFLOP/s",
                     "frac": (achieved / peak64) if peak64 else None, "traffic": traffic,
                     "peak_source": "measured in this run (rchem_peak_fma: DFMA chains on every SM); the "
                                    "bf16 tensor and HBM peaks of MEASURED_PEAKS.json do not bound this FP64 "
                                    "CUDA-core kernel",
                     "peak_fp32": peak32, "nominal_fp64": NOMINAL_FP64_TFLOPS,
                     "flops_per_build": st64["flops_fp64"], "hbm": hbm_context(traffic, ms)},
        "gpu_launches": launches * a.steps,
        "clocks": clocks,
        "wall_s_timed": wall,
        "cpu_baseline": cpu,
        "cpu_baseline_strong": cpu_strong,
        "targets": targets,
    }
    if rank == 0:
        print(json.dumps(line))
    b.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

"""Benchmark: direct-SCF Fock builds (J and K) per second on one GB300.

Workload (N=1): the (H2O)32 water cluster (seeded placement in a 14 A cube,
O-O >= 2.7 A) in the 6-31G*-shaped basis -- 608 Cartesian functions with
Cartesian d shells on O -- Schwarz threshold 1e-12: a full J+K build per step,
every unique shell quartet that passes the screen computed once.  The density
is the core-Hamiltonian guess density of that system (the work of a build does
not depend on the density's values).  ``--workload h2o8_631g`` runs the
(H2O)8 6-31G-shaped system instead.

Timing: W warm-up builds, then K timed builds, each bracketed by CUDA events
that the library records on the stream its kernels run on (from the copy of D
in to the copies of J and K out, so host submission latency is excluded); a
256 MiB buffer is written between timed builds (outside the events) so L2
(~126 MB) holds nothing of the previous build.  ``value`` is FP64 Fock
builds/s with D, J and K resident on the device; ``e2e`` is the same through
the C ABI with host arrays (H2D of D and D2H of J and K inside the timed
region, wall clock).  ``roofline`` is the dominant class kernel, timed alone
with CUDA events in this run, against the FP64 FMA peak measured in this run;
``roofline.build`` is the whole build.  ``forms`` holds the precision forms:
FP32 below fp32_tau = 1e-6 and 1e-4 with native FP64 above (the stated mixed
form; the Boys function of the FP32 quartets in FP64, or in FP32), and
double-float ("emulated FP64") above the threshold, each with its
converged-SCF energy and density against the FP64 SCF.

CPU baselines (rank 0, N=1): ``cpu_baseline`` is the reference's algorithm
(the JK_direct loops of src/basis.rs:383-428 over the THO integrals of
libpyquante2/cints.c with its own Boys function) on a bounded sample of the
build's n^4 index quadruples, all host threads; ``cpu_baseline_strong`` is a
strong CPU code over the same integrals (8-fold symmetry, the same Schwarz
screen, OpenMP) on a strided sample of bra pairs, extrapolated by the
integral count.

--impl reference: the reference's algorithm as above, on the same workload
and config, all host threads, each step a bounded sample extrapolated to a
whole build.
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

WORKLOAD = "h2o32_631gs"
DESCRIPTIONS = {
    "h2o32_631gs": "(H2O)32 water cluster (14 A cube), 6-31G*-shaped basis (608 Cartesian functions, Cartesian d "
                   "on O), direct-SCF J+K Fock build",
    "h2o8_631g": "(H2O)8 water cluster (9 A cube), 6-31G-shaped basis (104 Cartesian functions), direct-SCF J+K "
                 "Fock build",
    "h2o4_631gss": "(H2O)4 water cluster (4.5 A cube), 6-31G**-shaped basis (100 Cartesian functions), direct-SCF "
                   "J+K Fock build",
    "h2o_sto3g": "one water, STO-3G-shaped basis (7 functions), direct-SCF J+K Fock build",
}
METRIC = "Fock builds/s"
NOMINAL_FP64_TFLOPS = 1.25
SCHWARZ_TAU = 1e-12


def _args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default=WORKLOAD, choices=sorted(DESCRIPTIONS))
    ap.add_argument("--cpu-sample", type=int, default=0,
                    help="index quadruples per CPU reference step (0: sized to about 8-10 s of work)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-targets", action="store_true",
                    help="skip the (H2O)8, 512-geometry batch and gradient measurements")
    return ap.parse_args()


def _dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload_config(name):
    """The ``config`` object of the JSON line: the same for both arms (no GPU
    needed to form it)."""
    import rchem_gb300 as rc

    bname, Z, R = rc.geometry.config(name)
    return {"workload": name, "description": DESCRIPTIONS[name], "basis": bname,
            "basis_data": "fitted stand-in with the published shell structure and sizes "
                          "(rchem_gb300/basis_sets/make_basis_sets.py), not the published exponents",
            "nbf": rc.expand_shells(Z, bname).nbf, "natoms": int(len(Z)), "schwarz_tau": SCHWARZ_TAU,
            "density": "core-Hamiltonian guess density",
            "l2": "256 MiB buffer written between timed GPU steps (outside the timed events)"}


def core_guess_density(rc, b, nocc):
    S = rc.S(b)
    H = rc.T(b) + rc.V(b)
    w, U = np.linalg.eigh(S)
    X = U @ np.diag(w ** -0.5) @ U.T
    _, Cp = np.linalg.eigh(X.T @ H @ X)
    C = X @ Cp
    return C[:, :nocc] @ C[:, :nocc].T, H


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region,
    of the GPU this process runs on (selected by its UUID or PCI bus id:
    nvidia-smi numbers GPUs physically and ignores CUDA_VISIBLE_DEVICES)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.gpu_id = self.device_id(device)
        self.proc = None
        self.lines = []

    @staticmethod
    def device_id(device):
        try:
            import torch

            p = torch.cuda.get_device_properties(device)
            uuid = getattr(p, "uuid", None)
            if uuid is not None:
                s = str(uuid)
                return s if s.startswith("GPU-") else "GPU-" + s
            if hasattr(p, "pci_bus_id"):
                return "%08X:%02X:%02X.0" % (getattr(p, "pci_domain_id", 0), p.pci_bus_id, p.pci_device_id)
        except Exception:  # noqa: BLE001 -- no id: fall back to the visible index
            pass
        return str(device)

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", self.gpu_id, "--query-gpu=" + self.Q,
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
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "gpu": self.gpu_id}
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
                "samples": len(sm), "gpu": self.gpu_id}


def _oracle_basis(workload):
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    import rchem_gb300 as rc

    bname, Z, R = rc.geometry.config(workload)
    return O, O.expand_basis(Z, R, rc.load_bse(bname))


def cpu_reference_rate(workload, sample=0, steps=1, target_s=10.0, seed=17):
    """The reference's JK_direct loops (src/basis.rs:383-428: for every
    (mu, nu, lambda, sigma) and every primitive quartet, two THO ERIs with the
    shipped Boys function) on seeded random index quadruples, all host
    threads.  A whole build is the sum of the blocks of all n^4 quadruples,
    so builds/s = sampled quadruples / (time * n^4).  ``sample`` = 0 sizes the
    sample from a pilot so that each step takes about ``target_s`` seconds.
    Returns (rates, threads, quadruples per step, n)."""
    O, ob = _oracle_basis(workload)
    port = O.port()
    port.set_boys(False)
    try:
        threads = port.num_threads()
        n = ob.n
        rng = np.random.default_rng(seed)
        X = rng.normal(size=(n, n))
        D = X @ X.T / n
        m = sample
        if not m:
            pm = 64 * threads
            q = rng.integers(0, n, size=(4, pm))
            t0 = time.perf_counter()
            O.JK_direct_quartets(ob, D, *q)
            per = max(time.perf_counter() - t0, 1e-6) / pm
            m = int(min(max(threads, target_s / per), 2e8))
        rates = []
        for _ in range(steps):
            q = rng.integers(0, n, size=(4, m))
            t0 = time.perf_counter()
            O.JK_direct_quartets(ob, D, *q)
            dt = time.perf_counter() - t0
            rates.append(m / (dt * float(n) ** 4))
    finally:
        port.set_boys(True)
    return rates, threads, m, n


def cpu_strong_rate(workload, D, tau=SCHWARZ_TAU, target_s=8.0, target_1core_s=4.0):
    """A strong CPU Fock build with the reference's own integrals (THO ERIs,
    the shipped Boys function): each unique contracted integral once (8-fold
    symmetry), quartets with Q_ij Q_kl < tau skipped like the GPU build,
    OpenMP over bra pairs.  All threads and one core are each timed on a
    strided sample of the bra pairs sized to about ``target_s`` /
    ``target_1core_s`` seconds (the whole build when it fits) and extrapolated
    by the number of integrals that pass the screen."""
    O, ob = _oracle_basis(workload)
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
        pilot = np.arange(0, npair, 97)
        t0 = time.perf_counter()
        c_p = O.JK_sym_screened(ob, D, Q, tau, pairs=pilot)[2]
        per_int_all = (time.perf_counter() - t0) / max(c_p, 1)

        def sampled(per_int, target, nthreads):
            stride = int(min(max(1, round(total * per_int / target)), npair))
            sample = np.arange(stride // 2, npair, stride) if stride > 1 else None
            t0 = time.perf_counter()
            c = O.JK_sym_screened(ob, D, Q, tau, pairs=sample, nthreads=nthreads)[2]
            t = time.perf_counter() - t0
            desc = ("one whole build (%d integrals)" % c if sample is None else
                    "%d of %d bra pairs (every %d-th), %d integrals, extrapolated to the %d of a build"
                    % (len(sample), npair, stride, c, total))
            return c / (t * total), desc

        v_all, d_all = sampled(per_int_all, target_s, 0)
        v_1, d_1 = sampled(per_int_all * threads, target_1core_s, 1)
    finally:
        port.set_boys(True)
    return {"value": v_all, "unit": "builds/s", "cores": threads, "kind": "port",
            "algorithm": "each unique contracted integral once (8-fold symmetry), Schwarz screen Q_ij Q_kl >= %g "
                         "over contracted functions, THO ERIs of libpyquante2/cints.c with the shipped Boys "
                         "function, OpenMP dynamic over bra pairs" % tau,
            "sample": d_all, "schwarz_s": t_q, "integrals_per_build": total,
            "one_core": {"value": v_1, "unit": "builds/s", "cores": 1, "sample": d_1}}


def peak_fma(lib):
    import ctypes

    out = {}
    for bits in (64, 32):
        v = ctypes.c_double(0.0)
        out[bits] = v.value if lib.rchem_peak_fma(bits, ctypes.byref(v)) == 0 else None
    return out


def class_label(cl):
    s = "spd"
    return "(%s%s|%s%s)" % tuple(s[x] for x in cl)


def list_roofline(b, peak64, traffic_map=None, emulated=False):
    """Each class list of the current FP64 plan timed alone (CUDA events on the
    handle's stream; the fastest of three passes, so a transient slowdown of
    the shared machine does not pick the dominant list): algorithmic FLOPs per
    launch / launch time.  Returns the dominant list's roofline and the
    per-list table."""
    passes = [b.list_times(SCHWARZ_TAU, 0.0, emulated=emulated) for _ in range(3)]
    times = [(k, (min(p[i][1][0] for p in passes), 0.0)) for i, (k, _) in enumerate(passes[0])]
    cs = b.class_stats()
    rows = []
    for k, (ms64, _) in times:
        if ms64 <= 0.0:
            continue
        fl = cs[k]["flops"][0]
        rows.append({"kernel": "class %s FP64 J/K" % class_label(cs[k]["class"]), "ms": ms64, "flops": fl,
                     "tflops": fl / (ms64 * 1e-3) / 1e12, "quartets": cs[k]["quartets"][0],
                     "prim_quartets": cs[k]["prim_quartets"][0]})
    rows.sort(key=lambda r: -r["ms"])
    top = rows[0]
    traffic = None
    if traffic_map:
        traffic = traffic_map.get(top["kernel"])
    frac = top["tflops"] / peak64 if peak64 else None
    return {"bound": "fp64", "kernel": top["kernel"], "achieved": top["tflops"], "peak": peak64, "unit": "TFLOP/s",
            "frac": frac, "traffic": traffic, "flops_per_launch": top["flops"], "launch_ms": top["ms"],
            "share_of_serial_time": top["ms"] / sum(r["ms"] for r in rows)}, rows


def _traffic(workload):
    tpath = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(tpath) as f:
            return json.load(f).get(workload) or {}
    except (OSError, ValueError):
        return {}


def fock_forms(rc, torch, b, J, K, Dh, J64, K64, run, steps, warmup, scf_ref):
    """The precision forms on the same workload: time, J/K at the timed
    density against FP64, and the converged SCF against the FP64 SCF."""
    out = {}
    # (tag, fp32_tau, emulated, FP32 quartets' Boys function: "fp32" | "rec64" | "boys64", description)
    forms = (("mixed_1e-6_rec64", 1e-6, False, "rec64",
              "FP32 for quartets with Q_ab Q_cd < 1e-6, their Boys-function downward recursion in FP64 (table "
              "values in FP32), native FP64 above, FP64 accumulation: the stated mixed form, literally"),
             ("mixed_1e-6_boys64", 1e-6, False, "boys64",
              "as mixed_1e-6_rec64 with the FP32 quartets' whole Boys function (table values too) in FP64"),
             ("mixed_1e-6", 1e-6, False, "fp32",
              "as mixed_1e-6_rec64 with the recursion in FP32 too (the Boys function's error, <= 2e-6 relative, "
              "is that of the FP32 argument)"),
             ("mixed_1e-4", 1e-4, False, "fp32", "as mixed_1e-6 with the FP32 threshold at 1e-4"),
             ("emulated", 0.0, True, "fp32",
              "double-float (hi+lo float pairs, ~48-bit significand) on the FP32 pipe for every quartet of the "
              "classes that have it, native FP64 for the rest: an addition beyond the stated form"),
             ("emulated_mixed_1e-6", 1e-6, True, "fp32",
              "FP32 below 1e-6, double-float above: an addition beyond the stated form"))
    ms64 = scf_ref["ms"]
    for tag, tau32, emul, bmode, what in forms:
        fl = {"fp32_boys64": bmode == "boys64", "fp32_rec64": bmode == "rec64"}
        b.autotune(SCHWARZ_TAU, tau32, emulated=emul, **fl)
        ms = float(np.mean(run(tau32, steps, warmup, emulated=emul, **fl)))
        st = b.stats()
        Jf, Kf = J.cpu().numpy(), K.cpu().numpy()
        t0 = time.perf_counter()
        r = rc.scf.rhf(b, thresh_e=1e-10, fp32_tau=tau32, emulated=emul, **fl)
        torch.cuda.synchronize()
        t_scf = time.perf_counter() - t0
        out[tag] = {
            "arithmetic": what, "fp32_tau": tau32, "emulated": emul, "fp32_boys": bmode, "ms": ms,
            "builds_per_s": 1000.0 / ms,
            "speedup_vs_fp64": ms64 / ms,
            "fp32_quartet_fraction": st["quartets_fp32"] / max(1, st["quartets_fp32"] + st["quartets_fp64"]),
            "dE_fixed_density_Eh": float(np.sum(Dh * (2 * (Jf - J64) - (Kf - K64)))),
            "max_abs_dJ": float(np.abs(Jf - J64).max()), "max_abs_dK": float(np.abs(Kf - K64).max()),
            "scf_dE_Eh": r["e_total"] - scf_ref["e_total"],
            "scf_max_abs_dD": float((r["D"] - scf_ref["D"]).abs().max()),
            "scf_iterations": r["iterations"], "scf_converged": r["converged"], "scf_s": t_scf}
    return out


def h2o8_target(rc, torch, lib_peak64):
    """The (H2O)8 6-31G-shaped Fock build (the smaller direct-SCF workload):
    FP64, mixed and emulated forms, CUDA events of the library, L2 flushed."""
    bname, Z, R = rc.geometry.config("h2o8_631g")
    nocc = int(sum(Z)) // 2
    out = {}
    with rc.Basis(Z, R, bname) as b:
        s = torch.cuda.Stream()
        b.set_stream(s.cuda_stream)
        Dh, _ = core_guess_density(rc, b, nocc)
        D = torch.from_numpy(Dh).cuda()
        J, K = torch.empty_like(D), torch.empty_like(D)
        flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
        for tag, tau32, emul in (("fp64", 0.0, False), ("mixed_1e-6", 1e-6, False), ("emulated", 0.0, True),
                                 ("emulated_mixed_1e-6", 1e-6, True)):
            b.autotune(SCHWARZ_TAU, tau32, emulated=emul)
            for _ in range(3):
                rc.JK_direct(J, K, b, D, fp32_tau=tau32, emulated=emul)
            ms = []
            for _ in range(20):
                with torch.cuda.stream(s):
                    flush.fill_(1)
                rc.JK_direct(J, K, b, D, fp32_tau=tau32, emulated=emul)
                ms.append(b.stats()["gpu_ms"])
            st = b.stats()
            m = float(np.mean(ms))
            out[tag] = {"ms": m, "builds_per_s": 1000.0 / m}
            if tag == "fp64":
                out[tag]["flops"] = st["flops_fp64"]
                out[tag]["build_tflops"] = st["flops_fp64"] / (m * 1e-3) / 1e12
                out[tag]["build_frac_of_fp64_peak"] = out[tag]["build_tflops"] / lib_peak64 if lib_peak64 else None
                out[tag]["quartets"] = st["quartets_fp64"]
            else:
                out[tag]["speedup_vs_fp64"] = out["fp64"]["ms"] / m
    return out


def other_targets(rc, torch):
    """The 512-geometry batch (energy + gradient) and the (H2O)4 6-31G**-shaped
    adjoint gradient."""
    out = {}
    geoms = rc.geometry.water_batch(512, seed=7)
    bb = rc.batch.BatchBasis(geoms, "6-31g-fit")
    rc.batch.rhf_native(bb, max_iter=2)  # warm-up (plans, graphs)
    rc.batch.rhf_batch(bb, max_iter=2)
    rec = {"geometries": bb.ngeom, "packed_elements": bb.packed, "sizes": sorted(set(bb.geom_nbf.tolist())),
           "scf_driver": "rchem_rhf (the whole SCF loop in the library)"}
    for tag, tau32, emul in (("fp64", 0.0, False), ("mixed", 1e-6, False), ("emulated_mixed", 1e-6, True)):
        bb.autotune(SCHWARZ_TAU, tau32, emulated=emul)
        # warm-up of this form's gradient (its work plan and graphs are built on first use)
        rc.batch.gradient_batch(bb, rc.batch.rhf_native(bb, max_iter=2, fp32_tau=tau32, emulated=emul),
                                fp32_tau=tau32, emulated=emul)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r = rc.batch.rhf_native(bb, thresh_e=1e-10, fp32_tau=tau32, emulated=emul)
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        rc.batch.gradient_batch(bb, r, fp32_tau=tau32, emulated=emul)
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
        bb.autotune(SCHWARZ_TAU, tau32, emulated=emul)
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
        b.autotune(SCHWARZ_TAU, 0.0)
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
        for tag, tau32, emul in (("mixed", 1e-6, False), ("emulated_mixed", 1e-6, True)):
            b.autotune(SCHWARZ_TAU, tau32, emulated=emul)
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
    # each step about 6 s of CPU work; the whole run (steps + one warm-up step) within about 2.5 minutes
    target = min(6.0, 150.0 / (steps + 1))
    cpu_reference_rate(a.workload, a.cpu_sample or 0, steps=1, target_s=0.2 * target)  # warm-up
    rates, threads, m, n = cpu_reference_rate(a.workload, a.cpu_sample, steps=steps, target_s=target)
    value = float(np.mean(rates))
    sample = ("%d seeded random (mu, nu, lambda, sigma) index quadruples per step of the %d^4 the JK_direct loops "
              "(src/basis.rs:392-425) visit, each block computed as those loops compute it (every primitive "
              "quartet, two THO ERIs of libpyquante2/cints.c with its own Numerical-Recipes Boys function); "
              "builds/s = quadruples / (time * n^4)" % (m, n))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "builds/s", "n_gpus": a.gpus,
        "steps": steps, "warmup": a.warmup, "ms_per_step": 1000.0 / value, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(a.workload),
        "cpu_baseline": {"value": value, "unit": "builds/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "builds/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "the reference is a Rust crate (no Rust toolchain here) over libpyquante2; its JK_direct "
                "algorithm runs as the C port in oracle/pq2_port.c (pinned bit-for-bit against the compiled "
                "libpyquante2), with shell coefficients taken by position so the d shells of this basis load",
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

    cfg = workload_config(a.workload)
    bname, Z, R = rc.geometry.config(a.workload)
    nocc = int(sum(Z)) // 2
    b = rc.Basis(Z, R, bname)
    n = b.nbf
    stream = torch.cuda.Stream()
    b.set_stream(stream.cuda_stream)
    Dh, H = core_guess_density(rc, b, nocc)
    tuned = b.autotune(SCHWARZ_TAU, 0.0)  # per-class tile shapes for this basis (one-time set-up)
    D = torch.from_numpy(Dh).cuda()
    J = torch.empty_like(D)
    K = torch.empty_like(D)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def run(tau32, steps, warmup, emulated=False, fp32_boys64=False, fp32_rec64=False):
        # device time of each build from the library's own CUDA events on the
        # stream its kernels run on (bracketing the copy of D in, the class
        # kernels and the copies of J and K out); the L2 flush runs before.
        for _ in range(warmup):
            rc.JK_direct(J, K, b, D, fp32_tau=tau32, emulated=emulated, fp32_boys64=fp32_boys64,
                         fp32_rec64=fp32_rec64)
        ms = []
        for _ in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(1)
            rc.JK_direct(J, K, b, D, fp32_tau=tau32, emulated=emulated, fp32_boys64=fp32_boys64,
                         fp32_rec64=fp32_rec64)
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
    if world > 1:
        torch.distributed.barrier()
    st64 = b.stats()
    J64, K64 = J.cpu().numpy(), K.cpu().numpy()
    ms = float(np.mean(ms64))
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    value = world * 1000.0 / ms

    # ---- end to end through the C ABI with host arrays ---------------------
    # D in, J and K out through pinned host buffers (numpy views of pinned
    # torch tensors): the library copies them on its own stream inside the call
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
    e2e_ms = float(np.mean(te)) * 1e3
    if world > 1:
        t = torch.tensor([e2e_ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_ms = float(t.item())
    e2e = world * 1000.0 / e2e_ms
    e2e_max_diff = max(float(np.abs(Jh - J64).max()), float(np.abs(Kh - K64).max()))

    # ---- roofline: the dominant class kernel on the FP64 FMA pipe -----------
    pk = peak_fma(_lib.lib())
    peak64, peak32 = pk[64], pk[32]
    traffic = _traffic(a.workload)
    roof, rows = list_roofline(b, peak64, traffic)
    build_tflops = st64["flops_fp64"] / (ms * 1e-3) / 1e12
    roof["peak_source"] = ("measured in this run (rchem_peak_fma: DFMA chains on every SM); the bf16 tensor and "
                           "HBM peaks of MEASURED_PEAKS.json do not bound this FP64 CUDA-core kernel")
    roof["peak_fp32"] = peak32
    roof["nominal_fp64"] = NOMINAL_FP64_TFLOPS
    roof["build"] = {"achieved": build_tflops, "frac": build_tflops / peak64 if peak64 else None,
                     "flops_per_build": st64["flops_fp64"], "ms": ms, "traffic": traffic.get("build")}
    roof["lists"] = rows

    # ---- precision forms (same timing), SCF against the FP64 SCF ----------
    forms = {}
    if rank == 0:
        # the first FP64 eigensolve of a process creates cuSOLVER's handle and
        # workspaces (about a second): do it before the SCF timings
        torch.linalg.eigh(torch.eye(n, dtype=torch.float64, device="cuda"))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r64 = rc.scf.rhf(b, thresh_e=1e-10)
        torch.cuda.synchronize()
        scf_ref = {"ms": ms, "e_total": r64["e_total"], "D": r64["D"]}
        forms = {"fp64": {"ms": ms, "builds_per_s": 1000.0 / ms, "quartets": st64["quartets_fp64"],
                          "eris": st64["eris_fp64"], "prim_quartets": st64["prim_quartets_fp64"],
                          "scf_e_total_Eh": r64["e_total"], "scf_iterations": r64["iterations"],
                          "scf_converged": r64["converged"], "scf_s": time.perf_counter() - t0}}
        forms.update(fock_forms(rc, torch, b, J, K, Dh, J64, K64, run, a.steps, a.warmup, scf_ref))

    # ---- CPU baselines (rank 0, N=1 only) ------------------------------------
    cpu, cpu_strong = None, None
    if rank == 0 and world == 1 and not a.no_cpu_baseline:
        rates, threads, m, _ = cpu_reference_rate(a.workload, a.cpu_sample, steps=1)
        cpu = {"value": rates[0], "unit": "builds/s", "cores": threads, "kind": "port",
               "sample": "%d seeded random (mu, nu, lambda, sigma) quadruples of the JK_direct loops "
                         "(src/basis.rs:392-425; THO ERIs, the shipped NR Boys function), builds/s = quadruples / "
                         "(time * %d^4)" % (m, n)}
        cpu_strong = cpu_strong_rate(a.workload, Dh)

    # ---- the other workloads (outside the headline timed region) -----------
    targets = None
    if rank == 0 and not a.no_targets:
        targets = {"h2o8_631g_fock": h2o8_target(rc, torch, peak64)}
        targets.update(other_targets(rc, torch))

    clocks = clk.summary()
    cls = [c["class"] for c in b.class_stats()]
    launches = st64["kernels"] + 1  # class kernels + symmetrise
    line = {
        "metric": METRIC, "value": value, "unit": "builds/s", "n_gpus": world, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic", "config": cfg,
        "tuning": "rchem_autotune per class list before timing (lanes per quartet; warp-cooperative kernel with "
                  "32, 16 or 8 lanes per quartet for the classes of total angular momentum >= 4: tile shape 0, -16, "
                  "-8)",
        "eris_per_s": st64["eris_fp64"] / (ms * 1e-3),
        "forms": forms,
        "e2e": {"value": e2e, "unit": "builds/s", "h2d_bytes_per_step": n * n * 8,
                "d2h_bytes_per_step": 2 * n * n * 8, "max_abs_diff_vs_device_build": e2e_max_diff},
        "roofline": roof,
        "gpu_launches": launches * a.steps,
        "clocks": clocks,
        "wall_s_timed": wall,
        "cpu_baseline": cpu,
        "cpu_baseline_strong": cpu_strong,
        "targets": targets,
        "tile_shapes_fp64": {class_label(cls[k]): v for (k, p), v in tuned.items() if p == 0},
    }
    if rank == 0:
        print(json.dumps(line))
    b.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

"""Sigma-vector benchmark of the two-site SU2U1 DMRG hot path on one GB300.

Workload: one H_eff.psi on the middle two sites (11, 12) of an L=24, N=24,
S=0 SU2U1 chemistry Hamiltonian (seeded synthetic integrals, diagonal in
[-3, -0.3] Eh), random normalised MPS at bond dimension m=1024, boundaries
built on the GPU from that MPS.  A step is one sigma vector.  The inputs
(boundaries: several GB) are larger than L2, so no flush is needed between
steps.

Prints one JSON line (see the keys below).  ``--impl reference`` times the
C++/OpenMP restatement of the reference algorithm (``oracle/sigma_ref.cpp``)
on the host cores, on the same problem (layouts from a committed fixture).
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

METRIC = "H_eff.psi TFLOP/s (sigma vector, L=24 N=24 S=0 SU2U1, m=1024, middle sites)"


def metric_name(L: int, m: int) -> str:
    """The sigma metric's name for the workload run (METRIC at the default sizes)."""
    return f"H_eff.psi TFLOP/s (sigma vector, L={L} N={L} S=0 SU2U1, m={m}, middle sites)"
UNIT = "TFLOP/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--precision", default="bf16x3", choices=["fp64", "tf32", "bf16x3", "bf16x2"])
    ap.add_argument("--sweep", action="store_true",
                    help="time one full two-site sweep (FP64 and BF16x3 sigma forms) instead of sigma calls")
    ap.add_argument("--jd-maxiter", type=int, default=10)
    ap.add_argument("--shadow", action="store_true",
                    help="--sweep: one mixed sweep with an FP64 shadow solve at every microiteration (precision check)")
    ap.add_argument("--nsweeps", type=int, default=1, help="--sweep: number of sweeps")
    ap.add_argument("--forms", default="", help="--sweep: comma-separated forms (fp64, mixed, mixed_parts, "
                    "fp64_parts, fp64_heev, mixed_heev; default fp64,mixed,mixed_parts)")
    ap.add_argument("--kernel-profile", action="store_true",
                    help="--sweep: run the forms under torch.profiler (CUDA activity) and report device seconds "
                         "and launches per kernel (timings of such a run are not benchmark values)")
    ap.add_argument("--plan-cache", type=int, default=0,
                    help="--sweep: sigma plans kept, keyed by layouts (0: the engine default of 2)")
    ap.add_argument("--ramp", default="", help="--sweep: bond dimension per sweep, e.g. 256,256,512,512,1024,1024")
    ap.add_argument("--no-images", action="store_true",
                    help="BF16x3: split operands inside the block-product kernel instead of pre-split images")
    ap.add_argument("--compare-steps", type=int, default=2, help="FP64 sigma calls timed for the comparison")
    ap.add_argument("--autotune", action="store_true",
                    help="time every sigma plan-shape candidate on the workload and report the choice")
    ap.add_argument("--batch", action="store_true",
                    help="32 independent L=12 problems: batched Davidson against separate solves")
    ap.add_argument("--adjoint", action="store_true",
                    help="converge an FP64 ground state and time the energy gradient dE/d(integrals)")
    ap.add_argument("--adjoint-large", action="store_true",
                    help="energy gradient at L=30, m=1024 with right environments recomputed from checkpoints")
    ap.add_argument("--state-average", type=int, default=0, metavar="K",
                    help="state-averaged sweep for K roots (L=20, N=20, S=0, m=512 unless --L/--m given)")
    ap.add_argument("--graph", action="store_true",
                    help="--state-average: replay each microiteration's merged sigma from a CUDA graph")
    ap.add_argument("--store-every", type=int, default=6,
                    help="--adjoint-large: keep every k-th right environment, recompute the others")
    ap.add_argument("--L", type=int, default=24)
    ap.add_argument("--m", type=int, default=1024)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--stage-times", action="store_true", default=True)
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    def __init__(self, index=0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm = []
        mx = None
        reasons = set()
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx = float(r[1])
                for name, v in zip(["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"],
                                   r[4:8]):
                    if v.lower() == "active":
                        reasons.add(name)
            except (ValueError, IndexError):
                pass
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def ctypes_status():
    import ctypes
    from qcmaquis_gb300 import native as N
    v = ctypes.c_int32(-1)
    N.check(N.lib().qcm_device_status(ctypes.byref(v)), "qcm_device_status")
    return v.value


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return json.load(f)
    return {}


def k1_k3_stream_bytes(plan, left_elems: int, right_elems: int) -> int:
    """Bytes the K1 and K3 stages of a BF16x3 sigma plan stream by design: their
    BF16 slice images written and read back once (2 x the image bytes of the two
    GEMM stages, each panel ceil(K/32) x 3 slices x G x 512 bytes), T written, and
    the ket, contr, sigma and both boundaries moved once in FP32 (4 bytes per
    element).  The unit the measured DRAM traffic of these stages is scaled by."""
    img = 0
    for si, kind in enumerate(plan.stage_kinds()):
        if kind != "gemm":
            continue
        end = 0
        for src_off, img_off, src_buf, ld, R, K, kcontig, G in plan.stage_images(si)["panels"].tolist():
            if img_off >= 0:
                end = max(end, img_off + ((K + 31) // 32) * 3 * G * 512)
        img += end
    s0, s1, s2 = plan.scratch
    return int(2 * img + 4 * (s0 + s1 + s2 + plan.out_elems + left_elems + right_elems))


def _traffic_summary(path):
    vals = {}
    with open(path) as f:
        for line in f:
            for key in ("traffic_bytes_k1_k3", "k1_k3_stream_bytes"):
                if line.startswith(key + " ="):
                    vals[key] = int(line.split("=")[1])
    return vals


def captured_traffic(L: int, m: int, stream_bytes: int):
    """DRAM bytes per sigma of the roofline kernel (K1 + K3 stages: image builds and
    tcgen05 products) from a committed ncu summary, and where they come from.

    The capture is of a smaller case of the same workload (the full one holds
    16 GB on the device), scaled by the ratio of the two workloads' design stream
    bytes (``k1_k3_stream_bytes``): measured traffic over stream bytes is 1.035
    at m=512 and 1.054 at m=1024, so the traffic grows in proportion to them.
    None if there is no summary."""
    import glob
    exact = os.path.join(ROOT, "profiles", f"sigma_bf16x3_L{L}_m{m}_traffic.md")
    cands = [exact] if os.path.exists(exact) else sorted(
        glob.glob(os.path.join(ROOT, "profiles", f"sigma_bf16x3_L{L}_m*_traffic.md")))
    for path in cands:
        v = _traffic_summary(path)
        if "traffic_bytes_k1_k3" in v and v.get("k1_k3_stream_bytes"):
            per = v["traffic_bytes_k1_k3"] / v["k1_k3_stream_bytes"]
            how = ("measured" if path == exact
                   else f"scaled by the design stream bytes of the K1 and K3 stages, {per:.3f} DRAM bytes each")
            return per * stream_bytes, f"{os.path.relpath(path, ROOT)} ({how})"
    return None, None


def dgemm_peak_tflops():
    """cuBLAS FP64 GEMM rate on this GPU, measured live (4096^3, best of 3)."""
    import torch
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    for _ in range(2):
        a @ b
    best = 1e9
    for _ in range(3):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        s.record()
        a @ b
        e.record()
        torch.cuda.synchronize()
        best = min(best, s.elapsed_time(e) / 1e3)
    return 2.0 * n ** 3 / best / 1e12


class CppSigmaBaseline:
    """The C++/OpenMP oracle sigma (``oracle/sigma_ref.cpp``: the reference's lbtm
    algorithm, OpenMP over the right MPO bonds, block products in the host's
    OpenBLAS) on this benchmark's exact problem: layouts and MPO tensor from the
    committed fixture ``oracle/fixtures/sigma_L{L}_m{m}.npz``, ket and boundary
    values seeded normal numbers (the work does not depend on them).  Loads
    nothing of the library."""

    def __init__(self, L: int, m: int, seed: int = 7):
        import numpy as np
        from oracle import cpu_sigma as CS
        path = os.path.join(ROOT, "oracle", "fixtures", f"sigma_L{L}_m{m}.npz")
        self.CS = CS
        self.inp = CS.SigmaInputs(dict(np.load(path)))
        rng = np.random.default_rng(seed)
        self.x = rng.standard_normal(self.inp.psi_size)
        self.Ld = rng.standard_normal(self.inp.L_size)
        self.Rd = rng.standard_normal(self.inp.R_size)
        self.L, self.m = L, m

    def run(self):
        t0 = time.perf_counter()
        _, work = self.CS.sigma(self.inp, self.x, self.Ld, self.Rd)
        return float(work[0] + work[1]), time.perf_counter() - t0, int(work[2])

    def describe(self, times, threads):
        return (f"C++17 -O3 -fopenmp oracle sigma (lbtm; OpenMP over the {self.inp.W.col_dim} right MPO bonds; "
                f"{self.CS.host_blas()[1]}), the full L={self.L} m={self.m} middle-site sigma per run, "
                f"{len(times)} runs, median {sorted(times)[len(times) // 2]:.2f} s, {threads} threads; layouts from "
                f"oracle/fixtures, seeded random values")


def cpu_oracle_sample(L: int, m: int, runs: int = 3):
    """The C++ oracle's full sigma on the host cores, median of ``runs`` runs."""
    b = CppSigmaBaseline(L, m)
    res = [b.run() for _ in range(runs)]
    times = [t for _, t, _ in res]
    med = sorted(times)[len(times) // 2]
    return {"value": res[0][0] / med / 1e12, "unit": UNIT, "cores": res[0][2], "kind": "port",
            "sample": b.describe(times, res[0][2]), "seconds_per_sigma": med}


def run_reference(args):
    """CPU arm: the reference's sigma algorithm restated in C++/OpenMP (the
    reference itself does not build here: Boost, GSL and HDF5 are absent) on the
    host cores, on this benchmark's problem; each step is one full sigma."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    b = CppSigmaBaseline(args.L, args.m)
    for _ in range(args.warmup):
        b.run()
    flops = dt = 0.0
    times, threads = [], 1
    for _ in range(args.steps):
        f, t, threads = b.run()
        flops += f
        dt += t
        times.append(t)
    value = flops / dt / 1e12
    cpu = {"value": value, "unit": UNIT, "cores": threads, "kind": "port", "sample": b.describe(times, threads)}
    line = {"impl": "reference", "metric": metric_name(args.L, args.m), "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (the benchmark's layouts from a committed fixture, seeded random values)",
            "config": {"workload": f"sigma vector H_eff.psi, L={args.L} N={args.L} S=0 SU2U1, middle sites, "
                                   f"m={args.m}", "L": args.L, "m": args.m, "l2": "CPU run"},
            "cpu_baseline": cpu,
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def run_sweep(args):
    """One full two-site sweep (2(L-2) microiterations: eigensolver, truncation,
    boundary update) at bond dimension m from the same random right-normalised
    MPS, in the FP64 form and in the BF16x3 sigma form; prints one JSON line."""
    import numpy as np
    import torch
    from qcmaquis_gb300.engine import DeviceMPSTensor
    from qcmaquis_gb300.integrals import synthetic_integral_map
    from qcmaquis_gb300.model import QCModel
    from qcmaquis_gb300.mpo import make_mpo
    from qcmaquis_gb300.native import make_ts_cache_fmpo
    from qcmaquis_gb300.mps import bond_indices, right_canonical_chain
    from qcmaquis_gb300.sweep import SweepParams, run_dmrg
    L, nelec = args.L, args.L
    t0 = time.time()
    model = QCModel(L, synthetic_integral_map(L, seed=1, diag_range=(-3.0, -0.3)), nelec)
    mpo = make_mpo(model)
    ts = make_ts_cache_fmpo(mpo, model.phys)
    ramp = [int(x) for x in args.ramp.split(",")] if args.ramp else None
    # the random start has the bond dimension of the first sweep
    bonds = bond_indices(L, model.phys, (nelec, 0), ramp[0] if ramp else args.m)
    sites, _ = right_canonical_chain(model.phys, bonds, L, 0, np.random.default_rng(7))
    setup = time.time() - t0
    out = {}
    nsweeps = len(ramp) if ramp else args.nsweeps
    # (name, sigma precision, boundary precision, truncation, per-part timing): the plain
    # FP64 form with the reference's default SVD truncation against the mixed form
    # (BF16x3 sigma vectors, everything else FP64) with the same truncation -- the
    # headline pair, both run as in production (the host plans the next site problem
    # while the device finishes the boundary update); the mixed form once more with
    # the device synchronised after each part, for its time breakdown; and, on request
    # (--forms), both forms with the density-matrix (heev, noise 0) truncation
    variants = (("fp64", 0, 0, "svd", False), ("mixed", 2, 0, "svd", False), ("mixed_parts", 2, 0, "svd", True),
                ("fp64_parts", 0, 0, "svd", True), ("fp64_heev", 0, 0, "heev", True),
                ("mixed_heev", 2, 0, "heev", True))
    if not args.forms:
        variants = tuple(v for v in variants if v[0] in ("fp64", "mixed", "mixed_parts"))
    if args.forms:
        keep = set(args.forms.split(","))
        variants = tuple(v for v in variants if v[0] in keep)
    if args.shadow:
        variants = (("mixed_shadowed", 2, 0, "svd", True),)
    for name, prec, bprec, trunc, time_parts in variants:
        mps = [DeviceMPSTensor.from_host(t) for t in sites]
        p = SweepParams(nsweeps=nsweeps, max_bond_dimension=args.m, sweep_bond_dimensions=ramp,
                        truncation_initial=1e-16, truncation_final=1e-16, ietl_jcd_tol=1e-7,
                        ietl_jcd_maxiter=args.jd_maxiter, twosite_truncation=trunc,
                        alpha_initial=0.0, alpha_main=0.0, alpha_final=0.0)
        torch.cuda.synchronize()
        t1 = time.time()
        shadow = None
        if args.shadow:
            from qcmaquis_gb300.engine import Engine
            shadow = Engine("cuda", precision=0)
        prof = None
        if args.kernel_profile:
            from torch.profiler import ProfilerActivity, profile
            prof = profile(activities=[ProfilerActivity.CUDA])
            prof.__enter__()
        rec, _ = run_dmrg(model, mpo, p, nelec, mps=mps, precision=prec, ts_mpo=ts, boundary_precision=bprec,
                          time_parts=time_parts, plan_cache=args.plan_cache, shadow=shadow)
        torch.cuda.synchronize()
        kernels = None
        if prof is not None:
            prof.__exit__(None, None, None)
            kernels = {}
            for a in prof.key_averages():
                dt = getattr(a, "self_device_time_total", None)
                if dt is None:
                    dt = getattr(a, "self_cuda_time_total", 0.0)
                if dt and dt > 0:
                    kernels[a.key.split("(")[0]] = [round(dt / 1e6, 4), int(a.count)]
        out[name] = {"sweep_s": rec.sweep_seconds[-1], "sweep_seconds": rec.sweep_seconds, "wall_s": time.time() - t1,
                     "energy": rec.sweep_energy[-1], "sweep_energies": rec.sweep_energy,
                     "last_micro_energy": rec.energies[-1], "sigma_calls": rec.sigma_calls,
                     "max_bond": max(rec.bond_dimension), "truncated_weight": rec.sweep_truncated_weight[-1],
                     "truncation": trunc, "seconds_by_part": rec.seconds,
                     "repeated_layouts": len(rec.layout_digests) - len(set(rec.layout_digests)),
                     "plan_hits": rec.plan_hits,
                     "boundary_plan_hits": rec.boundary_plan_hits,
                     "microiterations": len(rec.layout_digests),
                     # the metric's rates over the whole run: sweeps and sigma vectors per second
                     "sweeps_per_s": len(rec.sweep_seconds) / sum(rec.sweep_seconds),
                     "sigma_per_s": rec.sigma_calls / sum(rec.sweep_seconds)}
        if kernels is not None:
            out[name]["kernel_device_s"] = dict(sorted(kernels.items(), key=lambda kv: -kv[1][0]))
        if rec.shadow:
            sh = np.array(rec.shadow)
            out[name]["shadow"] = {
                "what": ("per microiteration: mixed Ritz value, FP64 Rayleigh quotient of the mixed eigenvector, "
                         "FP64 eigensolver from the same start (Eh)"),
                "max_abs_ritz_minus_fp64_eh": float(np.max(np.abs(sh[:, 0] - sh[:, 2]))),
                "max_abs_rayleigh_minus_fp64_eh": float(np.max(np.abs(sh[:, 1] - sh[:, 2]))),
                "median_abs_rayleigh_minus_fp64_eh": float(np.median(np.abs(sh[:, 1] - sh[:, 2]))),
                "max_rayleigh_above_fp64_eh": float(np.max(sh[:, 1] - sh[:, 2])),
                "energies": sh.tolist()}
        del mps
        torch.cuda.empty_cache()
    if "fp64" not in out or "mixed" not in out:
        print(json.dumps({"metric": "sweep s (subset of forms)", "runs": out, "setup_s": setup}))
        return
    f, b = out["fp64"], out["mixed"]
    dsweep = [abs(x - y) for x, y in zip(b["sweep_energies"], f["sweep_energies"])]
    line = {"metric": f"sweep s (two-site sweep, L={L} N={nelec} S=0 SU2U1, m={args.m})", "value": b["sweep_s"],
            "unit": "s", "higher_is_better": False, "n_gpus": 1,
            "dtype": ("bf16x3 sigma products (fp32 accumulation); fp64 boundaries, eigensolver algebra, "
                      "SVD truncation, storage"),
            "data": "synthetic (seeded integrals, random right-normalised MPS)",
            "config": {"workload": (f"{nsweeps} sweep(s) from a random MPS at m={ramp[0] if ramp else args.m}"
                                    + (f", bond dimensions per sweep {ramp}" if ramp else f", Mmax {args.m}")
                                    + f", Davidson tol 1e-7, maxiter {args.jd_maxiter}, cutoff 1e-16; value = "
                                    "last sweep of the mixed form"), "L": L, "m": args.m},
            "fp64_sweep_s": f["sweep_s"], "speedup_vs_fp64_gpu": f["sweep_s"] / b["sweep_s"],
            "energy_fp64": f["energy"], "energy_mixed": b["energy"], "delta_energy_eh": abs(b["energy"] - f["energy"]),
            "max_delta_sweep_energy_eh": max(dsweep), "runs": out, "setup_s": setup}
    print(json.dumps(line))


def run_adjoint(args):
    """Converged FP64 ground state at L (default 16), N = L, S=0, bond dimension m
    (default 512), then the gradient of the energy with respect to every unique
    integral through the native energy-gradient plans, checked against central
    differences (step 1e-5) of the fixed-MPS energy on 20 random integrals (the RDM
    checks are in the tests)."""
    import numpy as np
    import torch
    from qcmaquis_gb300.engine import DeviceMPSTensor, Engine
    from qcmaquis_gb300.gradient import energy_gradient
    from qcmaquis_gb300.integrals import synthetic_integral_map
    from qcmaquis_gb300.model import QCModel
    from qcmaquis_gb300.mpo import make_mpo
    from qcmaquis_gb300.native import make_ts_cache_fmpo
    from qcmaquis_gb300.mps import bond_indices, right_canonical_chain
    from qcmaquis_gb300.sweep import SweepParams, expval, overlap, run_dmrg
    L = 16 if args.L == 24 else args.L
    m = 512 if args.m == 1024 else args.m
    nelec = L
    t0 = time.time()
    ints = synthetic_integral_map(L, seed=4, diag_range=(-2.0, -0.5))
    model = QCModel(L, ints, nelec)
    mpo = make_mpo(model)
    ts = make_ts_cache_fmpo(mpo, model.phys)
    bonds = bond_indices(L, model.phys, (nelec, 0), m)
    sites, _ = right_canonical_chain(model.phys, bonds, L, 0, np.random.default_rng(7))
    mps = [DeviceMPSTensor.from_host(t) for t in sites]
    ramp = [min(m, 128), min(m, 256), m, m, m, m]
    p = SweepParams(nsweeps=len(ramp), max_bond_dimension=m, sweep_bond_dimensions=ramp, ietl_jcd_tol=1e-8,
                    ietl_jcd_maxiter=10)
    rec, mps = run_dmrg(model, mpo, p, nelec, mps=mps, ts_mpo=ts)
    t_conv = time.time() - t0
    torch.cuda.synchronize()
    eng = Engine("cuda:0")
    energy_gradient(model, mps, nelec, engine=eng)   # warm-up (plan builds are host work)
    torch.cuda.synchronize()
    t1 = time.time()
    res = energy_gradient(model, mps, nelec, engine=eng)
    torch.cuda.synchronize()
    t_grad = time.time() - t1
    # central differences of the fixed-MPS energy
    efull = Engine("cuda:0", hermitian=False)
    nrm = overlap(mps)

    def energy(d):
        mm = make_mpo(QCModel(L, d, nelec))
        return expval(mps, mm, efull, (nelec, 0)) / nrm + mm.core_energy
    keys = sorted(ints)
    rng = np.random.default_rng(7)
    fd_err, fd_rows = 0.0, []
    h = 1e-5
    for i in rng.choice(len(keys), 20, replace=False):
        u = keys[i]
        up, dn = dict(ints), dict(ints)
        up[u] += h
        dn[u] -= h
        fd = (energy(up) - energy(dn)) / (2 * h)
        fd_err = max(fd_err, abs(fd - res.d_integrals[u]) / max(1.0, abs(fd)))
        fd_rows.append([list(u), fd, res.d_integrals[u]])
    # the spin-free RDMs through the same plans, and the energy they imply
    from qcmaquis_gb300.integrals import synthetic_integrals
    from qcmaquis_gb300.rdm import measure_rdm
    torch.cuda.synchronize()
    t2 = time.time()
    rdm1 = measure_rdm(model, mps, nelec, rank=1, engine=eng)
    rdm2 = measure_rdm(model, mps, nelec, rank=2, engine=eng)
    torch.cuda.synchronize()
    t_rdm = time.time() - t2
    tmat, V, core = synthetic_integrals(L, 4, (-2.0, -0.5))
    g1 = np.zeros((L, L))
    for (p_, q_), v in rdm1.items():
        g1[p_, q_] = g1[q_, p_] = v
    G = np.zeros((L, L, L, L))
    for (i, j, k, l_), v in rdm2.items():
        # element (a,b,c,d) = chemist Gamma[b,c,a,d] = sum_st <a+_bs a+_at a_dt a_cs>;
        # the element's index images pqrs = rspq = qpsr = srqp fill the rest
        for a, b, c, d in ((i, j, k, l_), (k, l_, i, j), (j, i, l_, k), (l_, k, j, i)):
            G[b, c, a, d] = v
    e_rdm = core + float(np.sum(tmat * g1)) + 0.5 * float(np.sum(V * G))
    line = {"metric": f"adjoint dE/d(integrals) s (L={L} N={nelec} S=0 SU2U1, m={m}, all unique integrals)",
            "value": t_grad, "unit": "s", "higher_is_better": False, "n_gpus": 1, "dtype": "f64",
            "data": "synthetic integrals (seeded), converged from a random MPS",
            "config": {"workload": f"gradient of the FP64 ground-state energy, L={L}, m={m}, {len(ints)} integrals",
                       "L": L, "m": m, "ramp": ramp},
            "n_integrals": len(res.d_integrals), "energy": res.energy, "sweep_energy": rec.sweep_energy[-1],
            "energy_consistency_eh": abs(res.energy - rec.sweep_energy[-1]),
            "converge_s": t_conv, "gradient_site_s": res.site_seconds,
            "fd_max_rel_err_20_integrals": fd_err, "fd_samples": fd_rows,
            "rdm_s": t_rdm, "rdm1_elements": len(rdm1), "rdm2_elements": len(rdm2),
            "energy_from_rdms": e_rdm, "energy_from_rdms_err_eh": abs(e_rdm - res.energy),
            "rdm_check": ("tests/test_energy_gradient.py: LiH gradient vs exact-diagonalisation RDM sums and the "
                          "exact 2-RDM vs the reference's golden 2-RDM (dmrg/tests/test2.cpp:60-120)")}
    print(json.dumps(line))


def run_adjoint_large(args):
    """dE/d(integrals) for every unique integral at L=30, N=30, S=0, m=1024 (a random
    right-normalised MPS: the gradient of the energy functional at that state).  The
    right environments are recomputed from every k-th stored one; a second pass keeps
    them all, and the two gradients must agree bit for bit.  Reports both times, the
    peak device memory of both, and the spread of the per-site energies (every site's
    energy-gradient plan gives the same <Psi|H|Psi>)."""
    import numpy as np
    import torch
    from qcmaquis_gb300.engine import DeviceMPSTensor, Engine
    from qcmaquis_gb300.gradient import energy_gradient
    from qcmaquis_gb300.integrals import synthetic_integral_map
    from qcmaquis_gb300.model import QCModel
    from qcmaquis_gb300.mps import bond_indices, right_canonical_chain
    L, m = 30, 1024
    t0 = time.time()
    ints = synthetic_integral_map(L, seed=4)
    model = QCModel(L, ints, L)
    bonds = bond_indices(L, model.phys, (L, 0), m)
    sites, _ = right_canonical_chain(model.phys, bonds, L, 0, np.random.default_rng(7))
    eng = Engine("cuda:0")
    mps = [DeviceMPSTensor.from_host(t) for t in sites]
    setup = time.time() - t0
    runs = {}
    k = max(1, args.store_every)
    # the first pass warms the engine's workspaces, so that the two measured passes'
    # peaks compare the environments alone
    for kk in (k, 1, k):
        torch.cuda.synchronize()
        torch.cuda.reset_peak_memory_stats()
        base = torch.cuda.memory_allocated()
        stats = {}
        t1 = time.time()
        res = energy_gradient(model, mps, L, engine=eng, store_every=kk, stats=stats)
        torch.cuda.synchronize()
        runs[kk] = (time.time() - t1, torch.cuda.max_memory_allocated() - base, res, stats)
    t_k, peak_k, res_k, st_k = runs[k]
    t_1, peak_1, res_1, st_1 = runs[1]
    same = all(res_k.d_integrals[u] == res_1.d_integrals[u] for u in res_1.d_integrals)
    env = st_1["env_bytes"]
    line = {"metric": f"adjoint dE/d(integrals) s (L={L} N={L} S=0 SU2U1, m={m}, right environments "
                      f"recomputed from every {k}th)",
            "value": t_k, "unit": "s", "higher_is_better": False, "n_gpus": 1, "dtype": "f64",
            "data": "synthetic integrals (seeded), random right-normalised MPS at m=1024",
            "config": {"workload": f"gradient of the energy at a fixed MPS, L={L}, m={m}, "
                                   f"{len(ints)} integrals", "L": L, "m": m, "store_every": k},
            "n_integrals": len(res_k.d_integrals), "energy": res_k.energy, "setup_s": setup,
            "bitwise_equal_to_keep_all": bool(same),
            "peak_device_bytes": {"recomputed": int(peak_k), "keep_all": int(peak_1)},
            "seconds": {"recomputed": t_k, "keep_all": t_1},
            "resident_environments": {"recomputed": st_k["peak_resident_environments"],
                                      "keep_all": st_1["peak_resident_environments"]},
            "peak_environment_bytes": {"recomputed": int(st_k["peak_environment_bytes"]),
                                       "keep_all": int(st_1["peak_environment_bytes"])},
            "right_environment_bytes": {"sum": int(sum(env.values())), "largest": int(max(env.values()))},
            "mps_bytes": int(sum(t.data.numel() * 8 for t in mps)),
            "site_energy_spread": float(np.ptp(st_k["site_energies"]) / res_k.norm),
            "gradient_site_s": res_k.site_seconds}
    print(json.dumps(line))


def run_state_average(args):
    """One state-averaged two-site sweep for K roots at L=20, N=20, S=0, m=512 (seeded
    synthetic integrals, diagonal in [-2, -0.5] Eh; a random right-normalised start at
    m=512), BF16x3 sigma vectors (FP64 with --precision fp64), equal weights: the
    K roots' sigma vectors in one merged plan per Davidson step.  Reports the sweep
    time, the roots' FP64 energies, Davidson steps and merged sigma launches."""
    import numpy as np
    import torch
    from qcmaquis_gb300.engine import DeviceMPSTensor
    from qcmaquis_gb300.integrals import synthetic_integral_map
    from qcmaquis_gb300.model import QCModel
    from qcmaquis_gb300.mpo import make_mpo
    from qcmaquis_gb300.native import make_ts_cache_fmpo
    from qcmaquis_gb300.mps import bond_indices, right_canonical_chain
    from qcmaquis_gb300.state_average import run_sa_dmrg
    from qcmaquis_gb300.sweep import SweepParams
    L = 20 if args.L == 24 else args.L
    m = 512 if args.m == 1024 else args.m
    k = args.state_average
    prec = {"fp64": 0, "tf32": 1, "bf16x3": 2, "bf16x2": 3}[args.precision]
    t0 = time.time()
    model = QCModel(L, synthetic_integral_map(L, seed=2, diag_range=(-2.0, -0.5)), L)
    mpo = make_mpo(model)
    ts = make_ts_cache_fmpo(mpo, model.phys)
    bonds = bond_indices(L, model.phys, (L, 0), m)
    sites, _ = right_canonical_chain(model.phys, bonds, L, 0, np.random.default_rng(7))
    mps = [DeviceMPSTensor.from_host(t) for t in sites]
    setup = time.time() - t0
    p = SweepParams(nsweeps=max(1, args.nsweeps), max_bond_dimension=m, truncation_initial=1e-16,
                    truncation_final=1e-16, ietl_jcd_tol=1e-7, ietl_jcd_maxiter=args.jd_maxiter)
    torch.cuda.synchronize()
    t1 = time.time()
    rec, _, _, _ = run_sa_dmrg(model, mpo, p, L, 0, nroots=k, mps=mps, precision=prec, ts_mpo=ts,
                               use_graph=args.graph)
    torch.cuda.synchronize()
    line = {"metric": f"state-averaged sweep s ({k} roots, L={L} N={L} S=0 SU2U1, m={m})",
            "value": rec.sweep_seconds[-1], "unit": "s", "higher_is_better": False, "n_gpus": 1,
            "dtype": f"{args.precision} sigma products; fp64 boundaries, eigensolver algebra, SVD truncation",
            "data": "synthetic (seeded integrals, random right-normalised MPS)",
            "config": {"workload": f"{p.nsweeps} state-averaged sweep(s) from a random MPS at m={m}, {k} roots, "
                                   "equal weights, Davidson tol 1e-7", "L": L, "m": m, "roots": k,
                       "cuda_graph": bool(args.graph)},
            "sweep_seconds": rec.sweep_seconds, "wall_s": time.time() - t1, "setup_s": setup,
            "root_energies": [list(map(float, e)) for e in rec.sweep_energies],
            "davidson_steps": int(sum(rec.iterations)), "merged_sigma_launches": int(sum(rec.sigma_launches)),
            "microiterations": len(rec.iterations), "max_bond": int(max(rec.bond_dimension)),
            "truncated_weight": float(max(rec.truncated_weight))}
    print(json.dumps(line))


def run_batch(args):
    """32 independent L=12, N=12, S=0 problems (integral seeds 1..32, bond dimensions
    drawn from {64, 128, 256, 512} with seed 0), the middle two-site problem of each:
    one Davidson solve of all of them together (the merged sigma plan, one launch per
    stage, replayed from a CUDA graph) against 32 separate solves."""
    import numpy as np
    import torch
    from qcmaquis_gb300.batch import BatchedSigma, solve_jcd_batched
    from qcmaquis_gb300.engine import Engine, SiteProblem
    from qcmaquis_gb300.jd import solve_ietl_jcd
    from qcmaquis_gb300.workloads import build_sigma_host, upload_sigma_workload
    from qcmaquis_gb300 import native as N
    nprob, L = 32, 12
    ms = np.random.default_rng(0).choice([64, 128, 256, 512], size=nprob)
    t0 = time.time()
    prec = {"fp64": N.PREC_FP64, "tf32": N.PREC_TF32, "bf16x3": N.PREC_BF16X3, "bf16x2": N.PREC_BF16X2}[args.precision]
    eng = Engine("cuda:0", precision=prec)
    probs = []
    for k in range(nprob):
        w = upload_sigma_workload(build_sigma_host(L=L, nelec=L, m=int(ms[k]), seed=k + 1,
                                                   diag_range=(-2.0, -0.5)), eng)
        probs.append((w.psi, w.left, w.right, w.ts_mpo))
    bs = BatchedSigma(eng, probs)
    bs.capture()
    setup = time.time() - t0
    x0 = bs.pack([p[0].data for p in probs])
    tol, maxiter = 1e-8, 10
    # warm-up of both paths (plans of the separate solves are built here)
    solve_jcd_batched(bs, x0, tol, maxiter, use_graph=True)
    for ket, Lb, Rb, ts in probs:
        eng.plan_cache_size = nprob + 2
        eng.sigma_plan(ket, Lb, Rb, ts)
    torch.cuda.synchronize()
    t1 = time.time()
    theta_b, _, iters_b = solve_jcd_batched(bs, x0, tol, maxiter, use_graph=True)
    torch.cuda.synchronize()
    t_batched = time.time() - t1
    t2 = time.time()
    theta_s, iters_s = [], []
    for ket, Lb, Rb, ts in probs:
        th, _, it = solve_ietl_jcd(SiteProblem(eng, Lb, Rb, ts), ket, tol, maxiter)
        theta_s.append(th)
        iters_s.append(it)
    torch.cuda.synchronize()
    t_sep = time.time() - t2
    # one sigma of the whole batch: merged graph replay against 32 separate calls
    reps = 20
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        bs.apply_graph(x0)
    e1.record()
    torch.cuda.synchronize()
    sig_b = e0.elapsed_time(e1) / reps
    e0.record()
    for _ in range(reps):
        for ket, Lb, Rb, ts in probs:
            eng.site_hamil2(ket, Lb, Rb, ts)
    e1.record()
    torch.cuda.synchronize()
    sig_s = e0.elapsed_time(e1) / reps
    line = {"metric": "batched Davidson solve s (32 independent L=12 N=12 S=0 SU2U1 problems)",
            "value": t_batched, "unit": "s", "higher_is_better": False, "n_gpus": 1, "dtype": args.precision,
            "data": "synthetic integrals (seeds 1..32), random MPS",
            "config": {"workload": "middle two-site problem of each of 32 systems, m drawn from {64,128,256,512}",
                       "m": [int(x) for x in ms], "tol": tol, "maxiter": maxiter},
            "separate_solves_s": t_sep, "speedup_vs_separate": t_sep / t_batched,
            "sigma_batch_ms_graph": sig_b, "sigma_separate_ms": sig_s,
            "max_theta_diff": float(np.max(np.abs(np.array(theta_s) - theta_b))),
            "iterations_equal": bool(list(iters_b) == iters_s), "setup_s": setup}
    print(json.dumps(line))


def run_autotune(args):
    """The plan-shape autotuner on the sigma workload: every candidate (split_k_segs,
    dense_min_terms), then tile widths and the K1 schedule, timed; the choice against
    the defaults (32, 64, N tiles up to 128, round-robin K1)."""
    import torch
    from qcmaquis_gb300 import native as N
    from qcmaquis_gb300.autotune import Autotuner, shape_key
    from qcmaquis_gb300.engine import Engine
    from qcmaquis_gb300.workloads import build_sigma_host, upload_sigma_workload
    prec = {"fp64": N.PREC_FP64, "tf32": N.PREC_TF32, "bf16x3": N.PREC_BF16X3, "bf16x2": N.PREC_BF16X2}[args.precision]
    w = build_sigma_host(L=args.L, m=args.m, seed=1)
    eng = Engine("cuda:0", precision=prec)
    upload_sigma_workload(w, eng)
    tuner = Autotuner(reps=5)
    t0 = time.time()
    opts = tuner.choice(eng, w.psi, w.left, w.right, w.ts_mpo)
    t_tune = time.time() - t0
    key = shape_key(w.psi.layout, w.left.layout, w.right.layout, w.ts_mpo, prec)
    ms = tuner.table[key]["ms"]
    best = min(ms.values())
    line = {"metric": f"autotuned sigma ms (L={args.L} N={args.L} S=0 SU2U1, m={args.m}, middle sites)",
            "value": best, "unit": "ms", "higher_is_better": False, "n_gpus": 1,
            "dtype": args.precision, "data": "synthetic", "config": {"workload": "sigma vector, plan-shape autotuning",
                                                                      "L": args.L, "m": args.m},
            "choice": opts, "default_ms": ms["32,64"],
            "speedup_vs_default": ms["32,64"] / best, "candidates_ms": ms,
            "plan_build_s": tuner.table[key]["plan_s"], "tuning_s": t_tune}
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.sweep:
        return run_sweep(args)
    if args.adjoint:
        return run_adjoint(args)
    if args.adjoint_large:
        return run_adjoint_large(args)
    if args.state_average:
        return run_state_average(args)
    if args.batch:
        return run_batch(args)
    if args.autotune:
        return run_autotune(args)
    import numpy as np
    import torch
    from qcmaquis_gb300 import native as N
    from qcmaquis_gb300.engine import Engine
    from qcmaquis_gb300.workloads import build_sigma_host, upload_sigma_workload

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    prec = {"fp64": N.PREC_FP64, "tf32": N.PREC_TF32, "bf16x3": N.PREC_BF16X3, "bf16x2": N.PREC_BF16X2}[args.precision]

    t0 = time.time()
    w = build_sigma_host(L=args.L, m=args.m, seed=1 + rank * 0)
    eng = Engine(f"cuda:{local}", precision=prec, use_images=not args.no_images)
    upload_sigma_workload(w, eng)
    plan = eng.sigma_plan(w.psi, w.left, w.right, w.ts_mpo)
    setup_s = time.time() - t0
    flops = plan.gemm_flops + plan.axpy_flops
    k1_k3_bytes = k1_k3_stream_bytes(plan, w.left.layout.size, w.right.layout.size)
    out = torch.empty(plan.out_elems, dtype=torch.float64, device=eng.device)
    stream = torch.cuda.current_stream()

    for _ in range(args.warmup):
        eng.site_hamil2(w.psi, w.left, w.right, w.ts_mpo, out=out)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    launches0 = eng.launches
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        torch.cuda.nvtx.range_push("sigma")
        for _ in range(args.steps):
            eng.site_hamil2(w.psi, w.left, w.right, w.ts_mpo, out=out)
        torch.cuda.nvtx.range_pop()
        ev1.record(stream)
        torch.cuda.synchronize()
    t_step = ev0.elapsed_time(ev1) / 1e3 / args.steps
    gpu_launches = eng.launches - launches0
    if world > 1:
        tt = torch.tensor([t_step], device=eng.device)
        torch.distributed.all_reduce(tt, op=torch.distributed.ReduceOp.MAX)
        t_step = float(tt.item())

    # per-stage times (CUDA events on the launching stream), for the roofline
    kinds = plan.stage_kinds()
    stage_t = [0.0] * len(kinds)
    reps = max(2, min(args.steps, 5))
    for _ in range(reps):
        for si in range(len(kinds)):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            eng.run(plan, ket=w.psi.data, left=w.left, right=w.right, out=out, first=si, last=si)
            b.record(stream)
            torch.cuda.synchronize()
            stage_t[si] += a.elapsed_time(b) / 1e3 / reps
    gemm_t = sum(t for t, k in zip(stage_t, kinds) if k == "gemm")
    axpy_t = sum(t for t, k in zip(stage_t, kinds) if k == "axpy")

    # end to end through the public API: pinned host psi -> device, sigma, -> host
    host_in = torch.from_numpy(N.Layout.of(w.psi_host.data).pack(w.psi_host.data)).pin_memory()
    host_out = torch.empty(plan.out_elems, dtype=torch.float64).pin_memory()
    dev_in = torch.empty_like(w.psi.data)
    from qcmaquis_gb300.engine import DeviceMPSTensor
    ket = DeviceMPSTensor(w.psi.phys_i, w.psi.left_i, w.psi.right_i, w.psi.layout, dev_in)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        dev_in.copy_(host_in, non_blocking=True)
        eng.site_hamil2(ket, w.left, w.right, w.ts_mpo, out=out)
        host_out.copy_(out, non_blocking=True)
    e1.record(stream)
    torch.cuda.synchronize()
    t_e2e = e0.elapsed_time(e1) / 1e3 / args.steps

    # the same sigma in plain FP64 on the GPU: speedup and relative error of this precision
    compare = None
    if prec != N.PREC_FP64 and args.compare_steps > 0:
        ref = torch.empty_like(out)
        eng.site_hamil2(w.psi, w.left, w.right, w.ts_mpo, out=ref, precision=N.PREC_FP64)
        torch.cuda.synchronize()
        c0, c1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        c0.record(stream)
        for _ in range(args.compare_steps):
            eng.site_hamil2(w.psi, w.left, w.right, w.ts_mpo, out=ref, precision=N.PREC_FP64)
        c1.record(stream)
        torch.cuda.synchronize()
        t64 = c0.elapsed_time(c1) / 1e3 / args.compare_steps
        eng.site_hamil2(w.psi, w.left, w.right, w.ts_mpo, out=out)
        torch.cuda.synchronize()
        rel = float((torch.linalg.norm(out - ref) / torch.linalg.norm(ref)).item())
        e_ref = float(torch.dot(w.psi.data, ref).item())
        e_mix = float(torch.dot(w.psi.data, out).item())
        compare = {"fp64_ms_per_step": t64 * 1e3, "speedup_vs_fp64_gpu": t64 / t_step,
                   "sigma_rel_err_vs_fp64": rel, "rayleigh_quotient_err_eh": abs(e_mix - e_ref),
                   "fp64_tflops": flops / t64 / 1e12}
    st = ctypes_status()

    peaks = measured_peaks()
    if prec == N.PREC_FP64:
        peak = dgemm_peak_tflops()
        roof = {"bound": "tensor", "achieved": plan.gemm_flops / gemm_t / 1e12, "peak": peak, "unit": "TFLOP/s",
                "frac": plan.gemm_flops / gemm_t / 1e12 / peak, "traffic": None,
                "kernel": "gemm_f64_kernel (K1 + K3 grouped block products)",
                "peak_source": "cuBLAS FP64 DGEMM 4096^3 measured in this run (no FP64 entry in MEASURED_PEAKS.json)"}
    else:
        peak = peaks.get("bf16_tflops", 1900.0)
        nprod = 6 if prec == N.PREC_BF16X3 else (3 if prec == N.PREC_BF16X2 else 1)
        ach = plan.gemm_flops * nprod / gemm_t / 1e12
        traffic, tsrc = (captured_traffic(args.L, args.m, k1_k3_bytes) if (prec == N.PREC_BF16X3 and not args.no_images)
                         else (None, None))
        roof = {"bound": "tensor", "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
                "traffic": traffic,
                "traffic_source": (f"{tsrc}: ncu dram__bytes_read.sum + dram__bytes_write.sum over the K1 and K3 "
                                   "launches of one sigma") if traffic else None,
                "traffic_gbs": traffic / gemm_t / 1e9 if traffic else None,
                "kernel": ("tc_img_kernel + build_images_kernel (tcgen05 K1 + K3 block products from "
                           "bulk-copied BF16 slice images)" if (prec in (N.PREC_BF16X3, N.PREC_BF16X2)
                                                                 and not args.no_images)
                           else "tc_gemm_kernel (tcgen05 K1 + K3 grouped block products)"),
                "achieved_counts": f"{nprod} tensor-core products per FP64-equivalent product",
                "peak_source": "MEASURED_PEAKS.json bf16_tflops (burst)"}
    axpy_gbs = plan.axpy_bytes / axpy_t / 1e9 if axpy_t > 0 else None

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        try:
            cpu = cpu_oracle_sample(args.L, args.m)
        except Exception as e:  # the baseline must not hide the GPU line
            cpu = {"error": str(e)}
        if cpu and "seconds_per_sigma" in cpu:
            # like for like: this run's sigma on the GPU against the CPU oracle's, per form
            cpu["gpu_over_cpu_same_sigma"] = {args.precision: cpu["seconds_per_sigma"] / t_step}
            if compare:
                cpu["gpu_over_cpu_same_sigma"]["fp64"] = cpu["seconds_per_sigma"] / (compare["fp64_ms_per_step"] / 1e3)

    value = flops / t_step / 1e12 * world
    line = {
        "metric": metric_name(args.L, args.m), "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": True,
        "scaling": "weak" if world > 1 else "weak", "vs_baseline": None,
        "dtype": {"fp64": "f64", "tf32": "tf32", "bf16x3": "bf16x3", "bf16x2": "bf16x2"}[args.precision],
        "data": "synthetic (seeded integrals and random MPS; no dataset)",
        "config": {"workload": f"sigma vector H_eff.psi, L={args.L} N={args.L} S=0 SU2U1, middle sites "
                               f"({args.L // 2 - 1},{args.L // 2}), m={args.m}",
                   **w.describe(), "precision": args.precision,
                   "l2": "working set of one sigma (boundaries, T, contr, operand images: about 16 GB) far above L2; no flush",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "setup_s": round(setup_s, 1)},
        "e2e": {"value": flops / t_e2e / 1e12 * world, "unit": UNIT,
                "h2d_bytes_per_step": int(w.psi.data.numel() * 8), "d2h_bytes_per_step": int(plan.out_elems * 8)},
        "gpu_launches": int(gpu_launches),
        "roofline": roof,
        "stages_ms": {f"{i}:{k}": round(t * 1e3, 3) for i, (k, t) in enumerate(zip(kinds, stage_t))},
        # naive count: every axpy term reads its source and reads+writes its output
        # in FP64 (3 x 8 B per element-term); sources are shared across terms and
        # served from L2, so this is an element-term rate, not DRAM traffic
        "axpy_element_term_rate_gbs_naive": axpy_gbs,
        "work": {"gemm_flops": plan.gemm_flops, "axpy_flops": plan.axpy_flops, "axpy_bytes": plan.axpy_bytes,
                 "k1_k3_stream_bytes": k1_k3_bytes},
        "clocks": clk.summary(),
        "vs_fp64_gpu": compare,
        "device_status": st,
        "cpu_baseline": cpu,
    }
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()

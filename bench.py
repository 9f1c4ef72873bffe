"""Benchmark: time-to-SCF of FORGE's real-space Hartree-Fock loop on one GB300.

One step = one SCF iteration of the hot path (H(k) assembly for all k, batched eigen-solve of
eigenpairs 1..N/2+10, density-matrix projectors, sort / Fermi level, energies, mixing and Hartree
potential) with every array resident in HBM.

Timed region (CUDA events on the library's stream, cumulative from one start event): the starting
guess, then the SCF iterations until the first one whose mean-field residual is below --tol
(1e-6 eV) on refined eigenpairs; value = time-to-SCF = that event time.  The region ends there
(iterations after convergence would time a converged state), so `steps` is the number of timed
iterations; --steps K is the number after which an unconverged SCF stops once the --budget-s
wall-clock budget is spent (or at --itmax); config.converged says which.  Before the timed region,
W warm-up iterations run from the plain guess; the timed SCF then starts again from its own guess,
so the warm-up does not shorten it.

e2e: the same SCF again, end to end through the reference-facing C-ABI calls with pinned host
buffers, the way a Fortran host would drive it (forge_gpu_solve with host Potential / zFock in and
Bands, zEigenvectors, zFockBulk out; sort; Fermi level; forge_gpu_get_fock with P_new out;
forge_gpu_optimal_step; forge_gpu_mix_potential; forge_gpu_get_state with zFock, Density and
Potential out), wall-clock timed from the guess to the converging iteration.

Modes: fast = learned warm start + mixed-precision eigen-solve with the FP64-accurate eigenpair
refinement; mixed = plain guess + the same mixed path; plain = plain guess + FP64.  The mixer is
Anderson/Pulay (depth 6) unless --mixer oda (the reference's OptimalStep) or --mixer linear.

Workloads: 4 = 1.05 deg twisted bilayer, m=31, N=11908, 4x4 k, nu=+2, eps=10 (headline, default);
1 = m=10, N=1324, 12x12 k, nu=+2; 2 = m=20, N=5044, 8x8 k, nu=-2, eps=8; 0 = m=5, N=364, 6x6 k,
nu=0.  Inputs are synthetic by construction (the geometry and the model are generated from the
parameters); nothing is read from disk except the warm-start network weights.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

CONFIGS = {
    0: dict(ntheta=5, numk=6, nfilling=0.0, epsilon=10.0, name="tbg_m5_N364_6x6_nu0_eps10"),
    1: dict(ntheta=10, numk=12, nfilling=2.0, epsilon=10.0, name="tbg_m10_N1324_12x12_nu+2_eps10"),
    2: dict(ntheta=20, numk=8, nfilling=-2.0, epsilon=8.0, name="tbg_m20_N5044_8x8_nu-2_eps8"),
    4: dict(ntheta=31, numk=4, nfilling=2.0, epsilon=10.0, name="tbg_m31_N11908_4x4_nu+2_eps10_1.05deg"),
}
METRIC = "time-to-SCF (s) and SCF iters, 1.05deg TBG: net+mixed vs plain FP64, same accuracy"

# Plain FP64 GPU SCF runs measured to convergence with `--mode plain --converge` (Pulay depth 6,
# beta 0.7, corrected DegFactor).  They are reported in the labelled field plain_fp64_recorded and
# give the reference arm its iteration count; they never enter `value`.
PLAIN_FP64_RECORDED = {
    # 1.05 deg: a plain FP64 SCF (about 70 minutes) does not fit one GPU lease, so the count is that of
    # the FP64-equivalent trajectory (every mixed solve refined to FP64 accuracy: the same iterates
    # to 1e-9) and the time per iteration is the measured FP64 one
    "tbg_m31_N11908_4x4_nu+2_eps10_1.05deg": {
        "iterations": 11, "converged": None, "estimated": True, "final_residual": 4.19e-07,
        "ms_per_iter": 347800.0, "guess_s": 300.0, "time_to_scf_s": 300.0 + 11 * 347.8,
        "date": "2026-12-04",
        "command": "python bench.py --config 4 --mode mixed --oa-always --converge --itmax 30 (11 iterations "
                   "to 4.2e-7 eV); FP64 iteration time 347.6-348.1 s measured on GB300 by "
                   "python3 bench.py --gpus 1 --steps 20 --warmup 5 (FP64 iterations 22-25 of its run); "
                   "FP64 guess = one FP64 solve of the 16 k points (16 x 18.7 s, forge_gb300.eigbench)"},
    "tbg_m10_N1324_12x12_nu+2_eps10": {
        "iterations": 6, "time_to_scf_s": 36.1, "ms_per_iter": 5160.0, "converged": True,
        "final_residual": 1.0e-07, "date": "2026-12-03",
        "command": "python bench.py --config 1 --mode plain --converge"},
}

# DRAM traffic of the dominant kernels from ncu captures small enough for the profiler
# (dram__bytes_read.sum + dram__bytes_write.sum), per unit of the work model: per algorithmic byte
# for the streaming kernels, per algorithmic flop for the sliced residual product (its DRAM bytes
# are panel re-reads, which grow with the tile-K products, i.e. with the flops, not with the
# operand bytes).
NCU_TRAFFIC_RATIO = {
    "hemv": (1.044, "bytes", "ncu --set full of k_trd_hemv<float> at N=5044, column 1501 (n'=3543): 52.25 MB "
                             "read + 0.19 MB written against 50.23 MB algorithmic (trailing lower triangle, "
                             "complex64); python -m forge_gb300.eigbench --m 20 --precision mixed"),
    "oa_gemm": (0.01628, "flops", "ncu (SpeedOfLight, MemoryWorkloadAnalysis) of k_tc_gemm_tf32<OaWEpi, 8, 1> at "
                                  "N=5044, iu=2532, depth 4: 2.528 TB/s x 24.89 ms = 62.9 GB for one launch of "
                                  "3.865e12 slice-product flop; python bench.py --config 2 --numk 2 --mode mixed "
                                  "--oa-always --steps 1 --warmup 3 --no-e2e --no-cpu-baseline"),
}


ROOFED = {"assemble", "hemv", "her2k", "backtransform", "projector", "window", "energy", "lr_matvec", "mix",
          "refine", "oa_gemm"}
TENSOR_STAGES = {"her2k", "backtransform", "projector", "window", "oa_gemm"}


def roofline(kernels, mode, peaks):
    """The roofline object of the dominant stage with a throughput bound.  kernels: the library
    profiler's per-stage totals ({stage: {"ms", "launches", "bytes", "flops"}}, launches > 0);
    peaks: (hbm GB/s, bf16 TFLOP/s, source)."""
    hbm, bf16, src = peaks
    cand = [k for k in kernels if k in ROOFED]
    if not cand:
        return None
    dom = max(cand, key=lambda k: kernels[k]["ms"])
    d = kernels[dom]
    per_launch_ms = d["ms"] / d["launches"]
    if mode != "plain" and dom in TENSOR_STAGES:
        ach = d["flops"] / d["launches"] / (per_launch_ms * 1e-3) / 1e12
        roof = {"bound": "tensor", "achieved": ach, "peak": bf16, "unit": "TFLOP/s", "frac": ach / bf16}
    else:
        ach = d["bytes"] / d["launches"] / (per_launch_ms * 1e-3) / 1e9
        roof = {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm}
    alg = d["bytes"] / d["launches"]
    tr = NCU_TRAFFIC_RATIO.get(dom)
    units = (d["flops"] if tr and tr[1] == "flops" else d["bytes"]) / d["launches"]
    roof.update({"kernel": dom, "launches": d["launches"], "avg_launch_ms": per_launch_ms,
                 "algorithmic_bytes_per_launch": alg, "algorithmic_flops_per_launch": d["flops"] / d["launches"],
                 "peak_source": f"{src} (MEASURED_PEAKS.json)" if src == "measured" else src,
                 "traffic": tr[0] * units if tr else None,
                 "traffic_source": f"{tr[2]}; ratio {tr[0]} B per algorithmic {tr[1][:-1]} x this run's "
                                   f"algorithmic {tr[1]} per launch (scaled from the small capture)" if tr
                 else None})
    return roof


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), float(p["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region (reads only)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu: int):
        self.gpu = gpu
        self.samples = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.t.join(timeout=2)
        sm = [float(s[1]) for s in self.samples if len(s) > 8 and s[1].replace(".", "").isdigit()]
        mx = [float(s[2]) for s in self.samples if len(s) > 8 and s[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for s in self.samples:
            if len(s) > 8:
                for nm, v in zip(names, s[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def _pinned(shape, dtype):
    """numpy array in page-locked host memory (cudaHostAlloc) for the e2e copies."""
    rt = C.CDLL("libcudart.so")
    n = int(np.prod(shape)) * np.dtype(dtype).itemsize
    p = C.c_void_p()
    if rt.cudaHostAlloc(C.byref(p), C.c_size_t(n), 0) != 0:
        raise RuntimeError(f"cudaHostAlloc of {n} bytes failed")
    buf = (C.c_byte * n).from_address(p.value)
    return np.ndarray(shape, dtype=dtype, buffer=buf, order="F")


def _log(obj):
    print(json.dumps(obj), file=sys.stderr, flush=True)


def _make(args, cfg):
    import forge_gb300 as fg
    mixed = args.mode in ("fast", "mixed")
    S = fg.Setup(ntheta=cfg["ntheta"], numk=cfg["numk"], nfilling=cfg["nfilling"], epsilon=cfg["epsilon"],
                 degfactor_mode=args.degfactor, precision="mixed" if mixed else "fp64",
                 nenforceC3=1 if args.c3 else 0)
    hf = fg.HartreeFock(S)
    hf.set_mixing(args.mixer, args.mix_depth, args.mix_beta)
    if mixed:
        hf.set_refinement(args.rr_width)
        if not args.no_oa:
            # the eigenpair refinement once the SCF is within reach of the tolerance (latched), or
            # on every solve (--oa-always: the FP64-equivalent trajectory)
            hf.set_eigen_refinement(1 if args.oa_always else 2, args.oa_below, 0.0, args.oa_depth)
    hf.LongRangeInteraction(copy_out=False)
    hf.synchronize()
    return S, hf


def _guess(hf, S, mode):
    """Starting guess: the learned warm start with the first-iteration fallback rule (fast: returns
    the state after the chosen start's first SCF iteration and that iteration's report), or the
    reference's plain guess (no iteration)."""
    if mode == "fast":
        from forge_gb300 import warmstart
        E1, rep1, info = warmstart.start(hf, S)
        return list(E1), info, [rep1]
    E0, _ = hf.PlainGuess()
    return list(E0), {}, []


def scf_device(hf, S, args, n_steps, budget_s, t_start_wall, profile=False):
    """The device-resident SCF from its guess: n_steps iterations, then (if it has not converged)
    more until it converges, itmax or the wall-clock budget.  Returns the per-iteration records with
    cumulative CUDA-event times from the start of the guess."""
    hf.mark(0)
    E, ginfo, first = _guess(hf, S, args.mode)
    hf.mark(1)
    t_guess = hf.elapsed_ms(0, 1) / 1e3
    if profile:
        hf.profile(True)
    hist = []
    t_conv = None
    # the fast start already ran the first iteration of the chosen start (and of the other one):
    # it is iteration 1, charged with the whole start-up time
    for rep in first:
        hist.append({"iter": 1, "ms": t_guess * 1e3, "t_cum": t_guess, "residual": rep["residual"],
                     "TotalEnergy": rep["TotalEnergy"], "nPartOccStates": rep["nPartOccStates"],
                     "info": rep["info"], "refined": rep["refined"]})
        if _converged(args, rep):
            t_conv = t_guess
    launches0 = hf.lib.forge_gpu_launch_count()
    timed_info = {}
    while True:
        i = len(hist)
        # the SCF of the timed region ends at convergence (a time-to-solution: iterations after it
        # would time a converged state), after n_steps iterations if that comes first and the
        # budget is spent, or at itmax
        stop = t_conv is not None or i >= args.itmax or (i >= n_steps and time.time() - t_start_wall > budget_s)
        if stop:
            timed_info = {"launches": hf.lib.forge_gpu_launch_count() - launches0}
            if profile:
                timed_info["prof"] = hf.profile_read()
                hf.profile(False)
            break
        slot = 2 + (i % 60)
        _stall_latch(hf, args, hist)
        rep, E, info = hf.ScfIteration(E)
        hf.mark(slot)
        t_cum = hf.elapsed_ms(0, slot) / 1e3
        prev = hist[-1]["t_cum"] if hist else t_guess
        rec = {"iter": i + 1, "ms": (t_cum - prev) * 1e3, "t_cum": t_cum, "residual": rep["residual"],
               "TotalEnergy": rep["TotalEnergy"], "nPartOccStates": rep["nPartOccStates"], "info": info,
               "refined": rep["refined"]}
        hist.append(rec)
        _log({k: (round(v, 1) if k == "ms" else v) for k, v in rec.items() if k != "t_cum"})
        if t_conv is None and _converged(args, rep):
            t_conv = t_cum
    return dict(t_guess=t_guess, hist=hist, t_conv=t_conv, guess_info=ginfo, E=E, **timed_info)


def _converged(args, rep):
    """Below the tolerance, and (mixed modes with the refinement) on refined eigenpairs: the state is
    then the FP64 SCF's, not the FP32-accurate solve's."""
    refine = args.mode in ("fast", "mixed") and not args.no_oa
    return rep["residual"] < args.tol and (rep["refined"] == 1 or not refine)


def _stall_latch(hf, args, hist):
    """Mixed modes: refine every later solve once the residual stalls below --oa-stall (no new best by
    a factor 0.8 in three iterations), even if it never reaches --oa-below."""
    if args.mode not in ("fast", "mixed") or args.no_oa or len(hist) < 4 or hist[-1].get("refined"):
        return
    res = [h["residual"] for h in hist]
    if res[-1] < args.oa_stall and min(res[-3:]) > 0.8 * min(res[:-3]):
        hf.set_eigen_refinement(1, 0.0, 0.0, args.oa_depth)
        _log({"refinement": "latched on stall", "after_iter": len(hist), "residual": res[-1]})


def scf_e2e(hf, S, args, budget_s):
    """The SCF through the reference-facing C-ABI calls with pinned host buffers (wall clock)."""
    lib, ctx = hf.lib, hf.ctx
    N, Nk, numb = hf.N, hf.Nk, hf.numb
    Ph = _pinned((N, N, 4), np.complex128)
    Pn = _pinned((N, N, 4), np.complex128)
    FBh = _pinned((N, N, 4), np.complex128)
    Vh = _pinned((N,), np.float64)
    Dh = _pinned((N,), np.float64)
    Bh = _pinned((numb, Nk), np.float64)
    Zh = _pinned((N, numb, Nk), np.complex128)
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    h2d = Ph.nbytes + Vh.nbytes
    d2h = Bh.nbytes + Zh.nbytes + FBh.nbytes + Pn.nbytes + Ph.nbytes + Dh.nbytes + Vh.nbytes
    import forge_gb300.api as api
    hf.synchronize()
    t0 = time.perf_counter()
    E, _, first = _guess(hf, S, args.mode)
    api._check(lib.forge_gpu_get_state(ctx, ptr(Ph), ptr(Dh), ptr(Vh)))
    hist = []
    t_conv = None
    for rep in first:
        hist.append({"iter": 1, "t_cum": time.perf_counter() - t0, "residual": rep["residual"],
                     "refined": rep["refined"]})
        if _converged(args, rep):
            t_conv = hist[-1]["t_cum"]
    t_start = time.time()
    while len(hist) < args.itmax and time.time() - t_start < budget_s:
        _stall_latch(hf, args, hist)
        api._check(lib.forge_gpu_solve(ctx, ptr(Vh), ptr(Ph), ptr(Bh), ptr(Zh), ptr(FBh)), allow_info=True)
        api._check(lib.forge_gpu_sort_energies(ctx, None, None, None))
        nf, ef, no, npart, deg = hf.FermiLevel()
        api._check(lib.forge_gpu_get_fock(ctx, C.c_double(deg), no, npart, ptr(Pn)))
        step, E = hf.OptimalStep(E)
        dn, res = hf.MixPotential(step)
        api._check(lib.forge_gpu_get_state(ctx, ptr(Ph), ptr(Dh), ptr(Vh)))
        t = time.perf_counter() - t0
        refined = hf.last_solve_refined()
        hist.append({"iter": len(hist) + 1, "t_cum": t, "residual": res, "refined": refined})
        _log({"e2e_iter": len(hist), "t_cum_s": round(t, 2), "residual": res, "refined": refined})
        if _converged(args, {"residual": res, "refined": refined}):
            t_conv = t
            break
    return dict(hist=hist, t_conv=t_conv, h2d=h2d, d2h=d2h,
                per_iter_s=(hist[-1]["t_cum"] / len(hist)) if hist else None)


def run_ours(args, cfg):
    import forge_gb300 as fg
    from forge_gb300 import build as fbuild
    fbuild.build()
    t_wall0 = time.time()
    S, hf = _make(args, cfg)
    t_setup = time.time() - t_wall0
    # warm-up: W iterations from the plain guess, untimed (the timed SCF starts again from its guess)
    E, _ = hf.PlainGuess()
    E = list(E)
    for w in range(args.warmup):
        rep, E, _ = hf.ScfIteration(E)
        _log({"warmup_iter": w + 1, "residual": rep["residual"]})
    clocks = ClockSampler(int(os.environ.get("LOCAL_RANK", "0")))
    clocks.start()
    run = scf_device(hf, S, args, args.steps, args.budget_s, t_wall0, profile=True)
    clk = clocks.stop()
    hf.profile(False)
    # order parameters of the state the timed SCF ended on (device reduction over P(0))
    try:
        run["order_parameters"] = hf.OrderParameters()
    except Exception as e:  # a diagnostic: its failure must not cost the measured line
        run["order_parameters"] = {"error": str(e)}
    state = None
    if args.save_state:
        state = _state_summary(hf, S)
    e2e = None
    if not args.no_e2e:
        e2e = scf_e2e(hf, S, args, max(60.0, args.budget_s - (time.time() - t_wall0)))
    N, Nk = hf.N, hf.Nk
    hf.close()
    return dict(run=run, clocks=clk, e2e=e2e, t_setup=t_setup, N=N, Nk=Nk, state=state,
                wall_s=time.time() - t_wall0)


def _state_summary(hf, S):
    """Converged-state summary (energies, bands, site densities, potential, order parameters and
    P(R) on the short bonds) for comparing SCF runs that cannot share a 9 GB density matrix."""
    from forge_gb300 import warmstart
    P, dens, V = hf.GetState()
    bands = hf.GetBands()
    g = hf.geometry
    op = hf.OrderParameters()
    bonds = warmstart.bond_list(S, g)
    pb = P[bonds[:, 0], bonds[:, 1], bonds[:, 2]]
    return dict(dens=dens, V=V, bands=bands, order=np.array([op[k] for k in sorted(op)]),
                order_names=np.array(sorted(op)), bonds=bonds, P_bonds=pb)


def cpu_sample(cfg, n_max=2000):
    """Bounded CPU sample (the cpu_baseline leg): one SCF iteration of the oracle port estimated from
    one k point on the principal n_max x n_max block of the sites (H(k) with ft / fv per pair as the
    reference evaluates them, zheevr il=1..n/2+10, ZHERK bulk projector, one energy pass), each part
    scaled to N by its exact order (N^2 for the pair loops, N^3 for zheevr and the projector), times
    Nk (+ 3 energy passes)."""
    from oracle import forge_oracle as fo
    import forge_gb300 as fg
    g = fg.build_geometry(fg.Setup(ntheta=cfg["ntheta"], numk=cfg["numk"], nfilling=cfg["nfilling"],
                                   epsilon=cfg["epsilon"]))
    so = fo.Setup(ntheta=cfg["ntheta"], numk=cfg["numk"], nfilling=cfg["nfilling"], epsilon=cfg["epsilon"])
    return _cpu_k_point(fo, so, np.asarray(g.Coords), g.nUnitCell_1, g.nUnitCell_2, g.tn[:, 0], g.tn[:, 1],
                        g.MomentaValues[0, min(1, cfg["numk"] - 1)], n_max)


def _cpu_k_point(fo, so, coords, u1, u2, t1, t2, vk, n_max):
    import scipy.linalg.blas as blas
    lib = fo._clib()
    if lib is None:
        return None
    N = so.ndim
    Ns = min(N, n_max)
    X = np.ascontiguousarray(coords[:Ns])
    mdl = fo._model_struct(so)
    u1 = np.ascontiguousarray(u1, dtype=np.int64)
    u2 = np.ascontiguousarray(u2, dtype=np.int64)
    t1, t2 = np.ascontiguousarray(t1, dtype=np.float64), np.ascontiguousarray(t2, dtype=np.float64)
    vk = np.ascontiguousarray(vk, dtype=np.float64)
    rng = np.random.default_rng(0)
    P = np.zeros((Ns, Ns, 4), dtype=np.complex128, order="F")
    P[:, :, 0] = np.eye(Ns) * 0.5
    V = rng.standard_normal(Ns) * 0.01
    H = np.zeros((Ns, Ns), dtype=np.complex128, order="F")
    cores = os.cpu_count() or 1
    t0 = time.time()
    lib.fo_hamiltonian_k(C.c_int64(Ns), fo._ptr(X), fo._ptr(u1), fo._ptr(u2), fo._ptr(t1), fo._ptr(t2), C.byref(mdl),
                         C.c_double(so.alpha), fo._ptr(V), fo._ptr(P), fo._ptr(vk), fo._ptr(H))
    t_asm = time.time() - t0
    iu, nl = Ns // 2 + 10, Ns // 2 - 9
    t0 = time.time()
    w, Z = fo.eigh_lower(H, iu)
    t_eig = time.time() - t0
    del H
    t0 = time.time()
    occ = np.asfortranarray(np.conj(Z[:, :nl - 1]))
    Cb = blas.zherk(1.0, occ, lower=1)
    t_proj = time.time() - t0
    del Cb, occ, Z
    t0 = time.time()
    out = np.zeros(2)
    lib.fo_energies_kf(C.c_int64(Ns), fo._ptr(X), fo._ptr(u1), fo._ptr(u2), fo._ptr(t1), fo._ptr(t2), C.byref(mdl),
                       fo._ptr(P), fo._ptr(out))
    t_en = time.time() - t0
    f2, f3 = (N / Ns) ** 2, (N / Ns) ** 3
    parts = dict(assemble=t_asm * f2, zheevr=t_eig * f3, projector=t_proj * f3, energy=t_en * f2)
    measured = dict(assemble=t_asm, zheevr=t_eig, projector=t_proj, energy=t_en)
    t_iter = so.Nk * (parts["assemble"] + parts["zheevr"] + parts["projector"]) + 3 * parts["energy"]
    if Ns == N:
        how = (f"one full k point at N={N} (H(k) with ft/fv per pair, zheevr il=1..N/2+10, ZHERK bulk projector, "
               f"one energy pass; OpenMP/OpenBLAS on {cores} threads), x {so.Nk} k + 3 energy passes")
    else:
        how = (f"one k point on the principal {Ns} x {Ns} block of the N={N} sites (H(k) with ft/fv per pair, "
               f"zheevr il=1..{iu}, ZHERK projector, one energy pass; OpenMP/OpenBLAS on {cores} threads), "
               f"EXTRAPOLATED to N by (N/{Ns})^2 for the pair loops and (N/{Ns})^3 for zheevr and the projector, "
               f"x {so.Nk} k + 3 energy passes")
    return dict(t_iter=t_iter, cores=cores, parts=parts, measured=measured, sample=how, full=(Ns == N))


def _iterations_source(rec):
    if not rec:
        return "no plain FP64 record for this workload: value is null, ms_per_step is measured"
    kind = ("iteration count of the FP64-equivalent SCF trajectory (every mixed solve refined to FP64 "
            "accuracy), with the same mixer" if rec.get("estimated") else
            "measured iteration count of the plain FP64 GPU SCF with the same mixer")
    return f"{kind} ({rec['command']}, {rec['date']}); the time per iteration is this run's"


def run_reference(args, cfg):
    """The reference arm: the oracle port (the reference's CPU algorithm restated; the Fortran
    reference cannot be built here) on the host cores, one full-size k point, no GPU library."""
    from oracle import forge_oracle as fo
    so = fo.Setup(ntheta=cfg["ntheta"], numk=cfg["numk"], nfilling=cfg["nfilling"], epsilon=cfg["epsilon"])
    t0 = time.time()
    g = fo.build_geometry(so)
    t_geo = time.time() - t0
    tn = g.tn
    cs = _cpu_k_point(fo, so, np.asarray(g.coords), g.ucell1, g.ucell2, tn[0], tn[1], g.vk(min(1, so.Nk - 1)),
                      n_max=args.ref_n_max)
    if cs is None:
        return None
    rec = PLAIN_FP64_RECORDED.get(cfg["name"])
    iters = rec["iterations"] if rec else None
    return dict(cs=cs, iters=iters, rec=rec, t_geo=t_geo)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=4, choices=sorted(CONFIGS))
    ap.add_argument("--mode", default="fast", choices=["fast", "mixed", "plain"],
                    help="fast: learned warm start + mixed-precision eigen-solve with eigenpair refinement; "
                         "mixed: plain guess + the same; plain: plain guess + FP64")
    ap.add_argument("--mixer", default="pulay", choices=["pulay", "oda", "linear"],
                    help="linear: P = beta P_new + (1 - beta) P_in with beta = --mix-beta")
    ap.add_argument("--mix-depth", type=int, default=6)
    ap.add_argument("--mix-beta", type=float, default=0.7)
    ap.add_argument("--degfactor", default="corrected", choices=["corrected", "reference"])
    ap.add_argument("--tol", type=float, default=1e-6, help="mean-field residual (eV) that defines SCF")
    ap.add_argument("--itmax", type=int, default=40)
    ap.add_argument("--budget-s", type=float, default=1500.0,
                    help="wall-clock budget of the repo arm after which no further iteration starts")
    ap.add_argument("--converge", action="store_true",
                    help="record run: continue to --tol within --itmax (no e2e, no CPU sample)")
    ap.add_argument("--save-state", default="", help="npz path for the converged-state summary")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--rr-width", type=int, default=32)
    ap.add_argument("--no-oa", action="store_true", help="mixed modes without the eigenpair refinement")
    ap.add_argument("--oa-below", type=float, default=1.0,
                    help="mixed modes: residual (eV) below which every later solve is refined (default: "
                         "from the second iteration on; the first iterations of the two starts that the "
                         "fast mode compares run unrefined)")
    ap.add_argument("--oa-stall", type=float, default=1e-3,
                    help="mixed modes: refine every later solve once the residual stalls below this (eV)")
    ap.add_argument("--oa-depth", type=int, default=4)
    ap.add_argument("--oa-always", action="store_true", help="mixed modes: refine every solve")
    ap.add_argument("--ref-n-max", type=int, default=1 << 30,
                    help="reference arm: largest principal block timed (default: the full N)")
    ap.add_argument("--c3", action="store_true")
    ap.add_argument("--numk", type=int, default=0,
                    help="profiling cases only: override the workload's k grid (numk x numk)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.converge:
        # record run: no fixed K, the SCF stops at the tolerance (or itmax)
        args.steps = 0
        args.no_e2e = True
        args.no_cpu_baseline = True
        args.budget_s = max(args.budget_s, 1e9)
    cfg = dict(CONFIGS[args.config])
    if args.numk > 0:
        cfg["numk"] = args.numk
        cfg["name"] += f"_k{args.numk}x{args.numk}"
    if args.c3:
        if cfg["numk"] % 3:
            ap.error("--c3 needs a k grid with numk divisible by 3")
        cfg["name"] += "_c3"
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return
        r = run_reference(args, cfg)
        if r is None:
            print(json.dumps({"impl": "reference", "unavailable": "oracle C library not built"}))
            return
        cs = r["cs"]
        val = cs["t_iter"] * r["iters"] if r["iters"] else None
        line = {"metric": METRIC, "value": val, "unit": "s", "n_gpus": 0, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": cs["t_iter"] * 1e3, "higher_is_better": False,
                "impl": "reference", "dtype": "f64", "data": "synthetic",
                "config": {"workload": cfg["name"], "iters": r["iters"], "cpu_parts_s": cs["parts"],
                           "measured_s": cs["measured"], "geometry_s": r["t_geo"],
                           "iterations_source": _iterations_source(r["rec"])},
                "cpu_baseline": {"value": val, "unit": "s", "cores": cs["cores"], "kind": "port",
                                 "sample": cs["sample"]},
                "e2e": {"value": val, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "vs_baseline": None}
        print(json.dumps(line))
        return
    if world > 1:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", os.environ.get("LOCAL_RANK", "0"))
        import torch.distributed as dist
        dist.init_process_group("gloo")
    r = run_ours(args, cfg)
    run = r["run"]
    hist = run["hist"]
    K = len(hist)
    timed = hist
    step_ms = [h["ms"] for h in timed]
    t_iter = float(np.mean(step_ms)) / 1e3 if step_ms else float("nan")
    converged = run["t_conv"] is not None
    t_scf = run["t_conv"] if converged else (hist[-1]["t_cum"] if hist else run["t_guess"])
    iters = next((h["iter"] for h in hist if _converged(args, h)), len(hist))
    e2e = r["e2e"]
    t_e2e = (e2e["t_conv"] if e2e and e2e["t_conv"] is not None else
             (e2e["hist"][-1]["t_cum"] if e2e and e2e["hist"] else None))
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([t_iter, t_scf, t_e2e or 0.0], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_iter, t_scf = float(t[0]), float(t[1])
        t_e2e = float(t[2]) if t_e2e is not None else None
    if rank != 0:
        return
    prof = run.get("prof", {})
    kernels = {k: v for k, v in prof.items() if v["launches"] > 0}
    roof = roofline(kernels, args.mode, _peaks())
    line = {"metric": METRIC, "value": t_scf, "unit": "s", "n_gpus": world, "steps": K,
            "warmup": args.warmup, "ms_per_step": t_iter * 1e3, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.mode == "plain" else "f32+f64",
            "data": "synthetic",
            "config": {"workload": cfg["name"], "mode": args.mode, "degfactor": args.degfactor,
                       "mixer": {"pulay": f"pulay(depth={args.mix_depth},beta={args.mix_beta})",
                                 "linear": f"linear(beta={args.mix_beta})"}.get(args.mixer, "oda"),
                       "N": r["N"], "Nk": r["Nk"], "converged": converged,
                       "iters_to_scf": iters if converged else None, "iterations_run": len(hist),
                       "residual_tol_eV": args.tol, "final_residual": hist[-1]["residual"] if hist else None,
                       "residuals": [h["residual"] for h in hist],
                       "refined": [h["refined"] for h in hist],
                       "energies": [h["TotalEnergy"] for h in hist],
                       "energy_per_atom": hist[-1]["TotalEnergy"] / r["N"] if hist else None,
                       "order_parameters": run.get("order_parameters"),
                       "guess_s": run["t_guess"], "setup_s": r["t_setup"], **run["guess_info"],
                       "value_source": "CUDA events of this run: start of the guess to the end of the first "
                                       "iteration below the residual tolerance",
                       "parallelism": f"replicas{world}",
                       "l2": "inputs larger than L2 (H(k) batch >= 129 MB per step)"},
            "e2e": {"value": t_e2e, "unit": "s", "h2d_bytes_per_step": e2e["h2d"] if e2e else 0,
                    "d2h_bytes_per_step": e2e["d2h"] if e2e else 0,
                    "converged": bool(e2e and e2e["t_conv"] is not None),
                    "iterations": len(e2e["hist"]) if e2e else 0,
                    "per_iter_s": e2e["per_iter_s"] if e2e else None} if e2e else None,
            "roofline": roof,
            "gpu_launches": int(run.get("launches", 0)),
            "stage_ms_per_step": {k: v["ms"] / max(1, K) for k, v in kernels.items()},
            "clocks": r["clocks"],
            "consistency": {"wall_s": r["wall_s"]}}
    rec = PLAIN_FP64_RECORDED.get(cfg["name"])
    if rec:
        line["plain_fp64_recorded"] = rec
    if args.save_state and r["state"] is not None:
        np.savez_compressed(args.save_state, residuals=np.array([h["residual"] for h in hist]),
                            energies=np.array([h["TotalEnergy"] for h in hist]),
                            ms=np.array([h["ms"] for h in hist]), **r["state"])
    if not args.no_cpu_baseline and world == 1:
        cs = cpu_sample(cfg)
        if cs is not None:
            n_it = rec["iterations"] if rec else (iters if converged else None)
            line["cpu_baseline"] = {"value": cs["t_iter"] * n_it if n_it else None, "unit": "s",
                                    "cores": cs["cores"], "kind": "port", "iterations": n_it,
                                    "ms_per_iteration": cs["t_iter"] * 1e3,
                                    "sample": cs["sample"] + (f"; time-to-SCF = per-iteration time x {n_it} "
                                                              "iterations of the plain FP64 record" if rec else
                                                              f"; x {n_it} iterations of this run")}
    print(json.dumps(line))


if __name__ == "__main__":
    main()

#!/usr/bin/env python
"""Benchmark of the GB300 Dirac-Coulomb Fock build.

Workload (the configuration the headline metric is quoted on): the seeded
ERI-kernel microbenchmark, 2^20 random primitive shell quartets with
l_a..l_d uniform on {0..3}, exponents log-uniform on [0.05, 1e6], centres
uniform in a 10-bohr cube with 20% overlapping pairs, split evenly over the
LL|LL, LL|SS, SS|LL and SS|SS component classes.  One step digests every
quartet into the Coulomb (J) and exchange (K) matrices of the shell pool
(CLMMTG batch types 1 and 5), FP64.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line (rank 0).  --impl reference times the CPU
restatement of the reference (the Fortran reference cannot be compiled
here: no Fortran compiler on either machine) on all host cores.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "bertha-program_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "Fock-build ERI quartets/s"
UNIT = "quartets/s"
WORKLOAD = "eri-microbench: 2^20 random shell quartets, l<=3, LL/SS classes"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    p.add_argument("--quartets", type=int, default=1 << 20)
    p.add_argument("--seed", type=int, default=2024)
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--ref-quartets", type=int, default=131072,
                   help="quartets per step of the reference arm (a bounded sample)")
    p.add_argument("--no-h2o", action="store_true",
                   help="skip the other configurations (H2O builds and SCF, TlF builds, "
                        "batched atoms) reported beside the headline")
    p.add_argument("--precision", default="tc32", choices=["fp64", "df32", "tc32"],
                   help="precision of the headline value; the others are timed beside it")
    return p.parse_args()


def config(args):
    """The workload, identical in both arms' lines (per-run figures such as
    the quartets of a step live outside it)."""
    return {"workload": WORKLOAD, "seed": args.seed,
            "pool": "32 centres x 4 l x 2 exponents (256 shells, NDIM 4096)",
            "l2": "flushed between timed steps (256 MiB write)",
            "parallelism": f"replicas x{args.gpus}"}


# ---------------------------------------------------------------------------
# CPU timing of the restatement (oracle) on a bounded sample
# ---------------------------------------------------------------------------
def cpu_rate(basis, quarts, dent, seconds, nthreads):
    """Quartets/s of the CPU restatement: chunks of 2048 quartets of every
    component class in turn until `seconds` of digestion time are spent."""
    from oracle import oracle as orc
    O = orc.QuartetOracle(basis)
    n = basis.ndim
    gd = np.zeros((n, n), complex, order="F")
    gx = np.zeros((n, n), complex, order="F")
    chunk, off, tot, nq = 2048, 0, 0.0, 0
    nmax = min(len(q) for q in quarts.values())
    while tot < seconds and off < nmax:
        for cls, q in quarts.items():
            s = q[off:off + chunk]
            O.prepare(s, *cls)
            t0 = time.perf_counter()
            O.digest(s, *cls, dent, gd, gx, nthreads=nthreads)
            tot += time.perf_counter() - t0
            nq += len(s)
        off += chunk
    O.close()
    return nq / tot, nq, tot


def run_reference(args):
    """The reference arm: the CPU restatement of ERIFAST/CLMMTG (the Fortran
    reference cannot be built on either machine) on all host cores.  A step
    is a bounded sample of the workload, the same number of quartets every
    step (equal per component class, drawn from the workload's lists in
    order), sized so that the whole run stays within a few minutes;
    ms_per_step is the measured time of that sample."""
    from oracle import oracle as orc
    from berthagpu import deck, workloads
    basis = workloads.microbench_pool(seed=args.seed)
    quarts = workloads.microbench_quartets(basis, args.quartets, seed=args.seed)
    dent = deck.density(basis, seed=args.seed)
    cores = os.cpu_count() or 1
    n = basis.ndim
    O = orc.QuartetOracle(basis)
    gd = np.zeros((n, n), complex, order="F")
    gx = np.zeros((n, n), complex, order="F")
    per_class = max(512, int(args.ref_quartets) // len(quarts))
    sample = {cls: q[:per_class] for cls, q in quarts.items()}
    for cls, q in sample.items():
        O.prepare(q, *cls)
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        for cls, q in sample.items():
            O.digest(q, *cls, dent, gd, gx, nthreads=cores)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
    O.close()
    nq = sum(len(q) for q in sample.values())
    ms = 1e3 * float(np.mean(times))
    value = nq / (ms * 1e-3)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config(args), "impl": "reference", "quartets_per_step": nq,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{nq} quartets per step ({per_class} per component class, "
                                   f"the first of each class's list) of the "
                                   f"{args.quartets}-quartet workload"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) == 6:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4)
                          if r[2 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


# DRAM bytes per k_quartet launch of this workload: dram__bytes_read.sum +
# dram__bytes_write.sum of one `ncu --set full` capture of the LL|LL launch
# at 2^16 quartets (16384 per class: 0.637 GB read + 0.034 GB written),
# scaled by 16 to the full step's 262144-quartet launch (DRAM traffic grows
# with the quartet count: the E-coefficients of the pool's random pairs).
TRAFFIC_BYTES_PER_LAUNCH = 10.749e9


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of the
# k_quartet_tc launches of one 2^20-quartet step of this workload's
# distribution, from a one-pass ncu launch list of the run module's
# microbenchmark (profiles/k_quartet_tc_eri_microbench_launches.md: 42.19 GB
# over the step's launches).
TC_TRAFFIC_BYTES_PER_STEP = 42.19e9


def read_traffic():
    """DRAM bytes per k_quartet launch (see TRAFFIC_BYTES_PER_LAUNCH)."""
    return TRAFFIC_BYTES_PER_LAUNCH


def h2o_fock_build(torch, with_cpu):
    """The H2O Dirac-Coulomb configuration: one stage-3 Fock build
    (CALL CLMFAST) through the C ABI with host arrays, FP64 and split
    precision, and the CPU restatement on one core for comparison."""
    import berthagpu
    from berthagpu import deck
    b = deck.h2o_basis()
    dent = deck.density(b, seed=1)
    out = {"ndim": b.ndim, "shells": len(b.shells()), "ilev": 3,
           "density": "seeded random Hermitian PSD (DENSTY form)"}
    res = {}
    for prec in ("fp64", "df32", "tc32", "auto"):
        fb = berthagpu.FockBuilder(b)
        fb.set_precision(prec)
        fb.set_screening(1e-12)
        fb.clmfast(dent, 3)
        ts = []
        for _ in range(3):
            t0 = time.perf_counter()
            gd, gx = fb.clmfast(dent, 3)
            ts.append(time.perf_counter() - t0)
        fb.close()
        res[prec] = (gd, gx)
        out[f"{prec}_s"] = float(np.median(ts))
    e = {}
    for prec, (gd, gx) in res.items():
        e[prec] = (0.5 * np.sum(dent * gd).real, 0.5 * np.sum(dent * gx).real)
    out["energy_j_eh"], out["energy_k_eh"] = e["fp64"]
    out["screen"] = 1e-12
    for prec in ("df32", "tc32", "auto"):
        out[prec + "_energy_err_eh"] = float(max(abs(e[prec][0] - e["fp64"][0]),
                                                 abs(e[prec][1] - e["fp64"][1])))
    if with_cpu:
        from oracle import oracle as orc
        # the oracle is unscreened: compare the GPU's unscreened FP64 build
        fb = berthagpu.FockBuilder(b)
        res["fp64"] = fb.clmfast(dent, 3)
        fb.close()
        t0 = time.perf_counter()
        rd, rx = orc.clmfast(b, dent, 3)
        out["cpu_port_1core_s"] = time.perf_counter() - t0
        scale = max(np.abs(rd).max(), np.abs(rx).max())
        out["fp64_max_abs_vs_cpu"] = float(max(np.abs(res["fp64"][0] - rd).max(),
                                               np.abs(res["fp64"][1] - rx).max()))
        out["fp64_rel_vs_cpu"] = out["fp64_max_abs_vs_cpu"] / scale
    return out


def h2o_breit_build(torch):
    """The H2O molecule under the Dirac-Coulomb-Breit Hamiltonian: one
    stage-3 closed-shell Breit exchange build (CALL BRTFAST) on device
    arrays, FP64, timed with CUDA events on the launching stream, plus the
    same call through the host-array entry point."""
    import berthagpu
    from berthagpu import deck, workloads
    b0 = deck.h2o_basis()
    b = deck.Basis(xyz=b0.xyz, lmax=b0.lmax, nfn=b0.nfn, ex=b0.ex, hmlt=deck.HMLT["DHFB"],
                   isym=b0.isym, name="H2O")
    dent = deck.density(b, seed=1)
    n = b.ndim
    q1, q2 = workloads.breit_quartets(b)
    flops = workloads.breit_flops(b, q1) + workloads.breit_flops(b, q2)
    fb = berthagpu.FockBuilder(b)
    d_D = torch.from_numpy(np.ascontiguousarray(dent.T)).cuda()  # column-major view
    d_B = torch.zeros((n, n), dtype=torch.complex128, device="cuda")
    st = torch.cuda.current_stream()
    fb.brtfast_device(d_D.data_ptr(), d_B.data_ptr(), 3, n, st.cuda_stream)
    ms = []
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        fb.brtfast_device(d_D.data_ptr(), d_B.data_ptr(), 3, n, st.cuda_stream)
        e1.record(st)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    bx = d_B.cpu().numpy().T
    ts = []
    for _ in range(3):
        t0 = time.perf_counter()
        bx_h = fb.brtfast(dent, 3)
        ts.append(time.perf_counter() - t0)
    fb.close()
    t = float(np.median(ms)) * 1e-3
    return {"ndim": n, "hmlt": "DHFB", "ilev": 3,
            "quartets": int(len(q1) + len(q2)),
            "classes": {"LS|LS (ab>=cd, both orders digested)": int(len(q1)),
                        "LS|SL (one of each (ab|cd), (dc|ba) pair; also digested as SL|LS)":
                            int(len(q2))},
            "device_s": t, "quartets_per_s": (len(q1) + len(q2)) / t,
            "flops": flops, "tflops": flops / t / 1e12,
            "host_api_s": float(np.median(ts)),
            "host_vs_device_max_abs": float(np.abs(bx_h - bx).max()),
            "energy_bx_eh": float(0.5 * np.sum(dent * bx).real)}


def h2o_scf(torch):
    """The H2O Dirac-Coulomb SCF configuration: closed shell, Gaussian
    nuclei, Schwarz 1e-12, converged to |dE| < 1e-9 Eh from the bare-nucleus
    guess; every iteration's Fock build, eigensolve and DIIS on the GPU.
    Run with the FP64 and the split-precision Fock build; the difference of
    the converged total energies is the precision's energy error."""
    from berthagpu import deck
    from berthagpu.scf import DHFSCF
    b = deck.h2o_basis()
    # library loading and solver initialisation outside the timing: one
    # untimed iteration of the same SCF
    torch.backends.cuda.preferred_linalg_library("cusolver")
    warm = DHFSCF(b, nocc=10, precision="fp64", screen=1e-12, torch=torch)
    warm.run(max_iter=1)
    warm.close()
    torch.cuda.synchronize()
    out = {"molecule": "H2O", "ndim": b.ndim, "nocc": 10, "screen": 1e-12, "etol_eh": 1e-10,
           "density_change_tol": 1e-7}
    for prec in ("fp64", "df32", "auto"):
        scf = DHFSCF(b, nocc=10, precision=prec, screen=1e-12, torch=torch)
        r = scf.run(max_iter=60, etol=1e-10, dtol=1e-7)
        scf.close()
        out[prec] = {k: r[k] for k in ("energy", "iterations", "converged", "density_change",
                                       "commutator", "wall_s", "fock_s", "linalg_s", "oneel_s")}
    for prec in ("df32", "auto"):
        out[f"energy_{prec}_vs_fp64_eh"] = out[prec]["energy"] - out["fp64"]["energy"]
    return out


def _device_time(torch, fn, reps=1):
    """Median device time (s) of fn() on the current stream, CUDA events."""
    st = torch.cuda.current_stream()
    ms = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        fn(st.cuda_stream)
        e1.record(st)
        e1.synchronize()
        ms.append(e0.elapsed_time(e1))
    return float(np.median(ms)) * 1e-3


TLF_BUDGET = 5e-7  # Eh per build: Coulomb + Breit within 1 uEh


def tlf_builds(torch):
    """The TlF Dirac-Coulomb-Breit configuration (R = 3.94 bohr on z, Tl
    28s24p16d12f and F 14s9p3d even-tempered, Schwarz 1e-12, DIATOM: real
    digestion): the stage-3 Coulomb and Breit builds in FP64, in the
    tensor-core precision and in the autotuned mixed mode (per angular class
    and Schwarz-bound decade the fastest kernel within an error budget of
    5e-7 Eh per build, so that the Coulomb plus Breit error stays within the
    configuration's 1 uEh), on device arrays (seeded Hermitian density), each
    timed with CUDA events after a first call that builds the lists (and
    tunes)."""
    import berthagpu
    from berthagpu import deck
    b = deck.tlf_basis()
    dent = deck.density(b, seed=1, real=True)
    n = b.ndim
    d_D = torch.from_numpy(np.ascontiguousarray(dent.T)).cuda()
    J, K, B = (torch.zeros((n, n), dtype=torch.complex128, device="cuda") for _ in range(3))
    out = {"ndim": n, "shells": len(b.shells()), "hmlt": "DHFB", "screen": 1e-12, "ilev": 3,
           "error_budget_eh_per_build": TLF_BUDGET}
    for prec in ("fp64", "tc32", "auto"):
        fb = berthagpu.FockBuilder(b)
        fb.set_precision(prec)
        fb.set_screening(1e-12)
        if prec == "auto":
            fb.set_error_budget(TLF_BUDGET)
        t0 = time.perf_counter()
        fb.clmfast_device(d_D.data_ptr(), J.data_ptr(), K.data_ptr(), 3, n)
        torch.cuda.synchronize()
        first = time.perf_counter() - t0
        t = _device_time(torch, lambda s: fb.clmfast_device(d_D.data_ptr(), J.data_ptr(),
                                                           K.data_ptr(), 3, n, s))
        r = {"coulomb_first_call_s": first, "coulomb_device_s": t,
             "energy_j_eh": float(0.5 * torch.sum(d_D * J).real),
             "energy_k_eh": float(0.5 * torch.sum(d_D * K).real)}
        t0 = time.perf_counter()
        fb.brtfast_device(d_D.data_ptr(), B.data_ptr(), 3, n)
        torch.cuda.synchronize()
        r["breit_first_call_s"] = time.perf_counter() - t0
        r["breit_device_s"] = _device_time(torch, lambda s: fb.brtfast_device(
            d_D.data_ptr(), B.data_ptr(), 3, n, s))
        r["energy_bx_eh"] = float(0.5 * torch.sum(d_D * B).real)
        r["dcb_build_s"] = r["coulomb_device_s"] + r["breit_device_s"]
        if prec != "fp64":
            r["coulomb_kernels"] = fb.auto_stats()
            r["breit_kernels"] = fb.breit_stats()
        fb.close()
        out[prec] = r
    f = out["fp64"]
    for prec in ("tc32", "auto"):
        r = out[prec]
        r["speedup_vs_fp64"] = {"coulomb": f["coulomb_device_s"] / r["coulomb_device_s"],
                                "breit": f["breit_device_s"] / r["breit_device_s"],
                                "dcb": f["dcb_build_s"] / r["dcb_build_s"]}
        r["energy_error_vs_fp64_eh"] = {
            "j": r["energy_j_eh"] - f["energy_j_eh"], "k": r["energy_k_eh"] - f["energy_k_eh"],
            "bx": r["energy_bx_eh"] - f["energy_bx_eh"],
            "total_two_electron": (r["energy_j_eh"] - r["energy_k_eh"] - r["energy_bx_eh"])
            - (f["energy_j_eh"] - f["energy_k_eh"] - f["energy_bx_eh"])}
    # the precision's effect on a converged DCB total energy: the small TlF
    # case (same geometry, angular momenta and exponent range), both SCFs
    # converged in energy and density, and the precisions' total energies at
    # the FP64 SCF's converged density
    from berthagpu.scf import DHFSCF
    bs = deck.tlf_small_basis()
    scf = {"case": "TlF, Tl 7s6p4d3f / F 4s3p1d, DHFB", "ndim": bs.ndim, "nocc": 90,
           "guess": "bare nucleus, maximum overlap from iteration 3",
           "etol_eh": 1e-10, "density_change_tol": 1e-4}
    dens = {}
    for prec in ("fp64", "auto"):
        s_ = DHFSCF(bs, nocc=90, precision=prec, screen=1e-12, torch=torch)
        if prec == "auto":
            s_.backend.fb.set_error_budget(TLF_BUDGET)
        # (the energy settles to 1e-10 Eh while the density keeps moving at
        # a few 1e-5 along near-degenerate rotations)
        r = s_.run(max_iter=150, etol=1e-10, dtol=1e-4, mom=3, return_density=True)
        dens[prec] = r["density"]
        scf[prec] = {k: r[k] for k in ("energy", "iterations", "converged", "density_change",
                                       "commutator", "wall_s", "fock_s")}
        s_.close()
    scf["energy_auto_vs_fp64_eh"] = scf["auto"]["energy"] - scf["fp64"]["energy"]
    at = {}
    for prec in ("fp64", "auto", "tc32"):
        s_ = DHFSCF(bs, nocc=90, precision=prec, screen=1e-12, torch=torch)
        if prec == "auto":
            s_.backend.fb.set_error_budget(TLF_BUDGET)
        s_.energy_at(dens["fp64"])  # first build: lists and tuning
        at[prec] = s_.energy_at(dens["fp64"])
        s_.close()
    scf["energy_at_fp64_density"] = at
    # (the small case's classes fall below the tuner's sampling threshold,
    # so its autotuned build is FP64 throughout; tc32 shows the tensor
    # cores' effect on a converged DCB energy)
    scf["energy_auto_vs_fp64_at_shared_density_eh"] = at["auto"] - at["fp64"]
    scf["energy_tc32_vs_fp64_at_shared_density_eh"] = at["tc32"] - at["fp64"]
    out["scf_tlf_small"] = scf
    return out


def batched_atoms(torch):
    """The batched-atoms configuration: 96 closed-shell atoms (Z drawn,
    seeded, from the closed-shell atoms He..Rn; n_s = 8+Z/4, n_p = 6+Z/5,
    n_d = Z/12, n_f = Z/24 even-tempered functions, Dirac-Coulomb, Schwarz
    1e-12) in one batched Fock build (one launch per component class for all
    96, or per tuned run of classes), FP64 and autotuned mixed precision,
    timed with CUDA events; and the batched SCF of 96 atoms drawn from He..Ca
    (the lighter half of the table, so that the whole SCF stays within the
    benchmark's time) to |dE| < 1e-9 Eh per atom in both precisions."""
    from berthagpu import deck
    from berthagpu.fock import FockBatch, FockBuilder
    from berthagpu.scf import BatchedDHFSCF
    bases = deck.batched_atoms(96, seed=2024)
    zs = [int(b.znuc[0]) for b in bases]
    dens = [deck.density(b, seed=2024 + k, nocc=z, real=True) for k, (b, z) in enumerate(zip(bases, zs))]
    D = torch.from_numpy(np.concatenate([d.ravel(order="F") for d in dens])).cuda()
    J, K = torch.zeros_like(D), torch.zeros_like(D)
    out = {"atoms": 96, "ndim_min": min(b.ndim for b in bases),
           "ndim_max": max(b.ndim for b in bases), "ndim_total": sum(b.ndim for b in bases)}
    energies = {}
    for prec in ("fp64", "auto"):
        fbs = []
        for b in bases:
            fb = FockBuilder(b, racah1=False)
            fb.set_precision(prec)
            fb.set_screening(1e-12)
            fbs.append(fb)
        batch = FockBatch(fbs)
        for fb in fbs:
            fb.close()
        t0 = time.perf_counter()
        batch.clmfast_device(D.data_ptr(), J.data_ptr(), K.data_ptr(), 3)
        torch.cuda.synchronize()
        first = time.perf_counter() - t0
        t = _device_time(torch, lambda s: batch.clmfast_device(D.data_ptr(), J.data_ptr(),
                                                              K.data_ptr(), 3, s))
        nq = batch.quartets()
        r = {"first_call_s": first, "device_s": t, "quartets": nq, "quartets_per_s": nq / t,
             "launches": batch.launches()}
        if prec == "auto":
            r["auto"] = batch.auto_stats()
        Jh, Kh = J.cpu().numpy(), K.cpu().numpy()
        e, off = [], 0
        for d in dens:
            m = d.shape[0] * d.shape[0]
            e.append(0.5 * np.sum(d.ravel(order="F") * (Jh[off:off + m] - Kh[off:off + m])).real)
            off += m
        energies[prec] = np.array(e)
        batch.close()
        out["build_" + prec] = r
    out["build_auto_vs_fp64_energy_max_abs_eh"] = float(
        np.abs(energies["auto"] - energies["fp64"]).max())
    light = deck.batched_atoms(96, seed=2024, zset=[z for z in deck.CLOSED_SHELL_ATOMS if z <= 20])
    lz = [int(b.znuc[0]) for b in light]
    res = {}
    for prec in ("fp64", "auto"):
        s = BatchedDHFSCF(light, lz, precision=prec, screen=1e-12, torch=torch)
        r = s.run(etol=1e-9, max_iter=80)
        s.close()
        res[prec] = r
    de = np.abs(np.array(res["auto"]["energy"]) - np.array(res["fp64"]["energy"]))
    out["scf_light"] = {
        "atoms": 96, "z": sorted(set(lz)), "etol_eh": 1e-9,
        "fp64": {k: res["fp64"][k] for k in ("iterations", "wall_s", "fock_s", "linalg_s",
                                              "quartets_per_build")},
        "auto": {k: res["auto"][k] for k in ("iterations", "wall_s", "fock_s", "linalg_s")},
        "all_converged": bool(all(res["fp64"]["converged"]) and all(res["auto"]["converged"])),
        "energy_auto_vs_fp64_max_abs_eh": float(de.max()),
        "energy_fp64_by_z": {str(z): e for z, e in zip(lz, res["fp64"]["energy"])}}
    return out


def fp64_peak(torch):
    """FP64 peak of this GPU measured now: cuBLAS DGEMM, 4096^3, best of 5."""
    n = 4096
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    a @ b
    best = 0.0
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        a @ b
        e.record()
        e.synchronize()
        best = max(best, 2.0 * n ** 3 / (s.elapsed_time(e) * 1e-3) / 1e12)
    del a, b
    return best


def tf32_peak(torch):
    """Dense TF32 tensor-core peak of this GPU measured now: cuBLAS FP32 GEMM
    with TF32 allowed, 8192^3, best of 5."""
    n = 8192
    old = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = True
    a = torch.randn(n, n, dtype=torch.float32, device="cuda")
    b = torch.randn(n, n, dtype=torch.float32, device="cuda")
    a @ b
    best = 0.0
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        a @ b
        e.record()
        e.synchronize()
        best = max(best, 2.0 * n ** 3 / (s.elapsed_time(e) * 1e-3) / 1e12)
    torch.backends.cuda.matmul.allow_tf32 = old
    del a, b
    return best


PATHS = ("fp64", "df32", "tc32")
DTYPE = {"fp64": "f64",
         "df32": "f32x2 double-float contractions; f64 Boys, R, J/K sums",
         "tc32": "tf32x3 tcgen05 contractions (fp32 accumulate); f64 Boys, R, J/K sums"}


def run_gpu(args):
    import torch
    import torch.distributed as dist

    import berthagpu
    from berthagpu import _lib, deck, replicas, workloads
    from berthagpu.build import build as build_lib

    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    if rank == 0:
        build_lib()
    if world > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
        dist.barrier()
        build_lib()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    basis = workloads.microbench_pool(seed=args.seed)
    raw = workloads.microbench_quartets(basis, args.quartets, seed=args.seed)
    # each component class's list grouped by angular class (CLMFAST's L-block
    # order); the segment table lets the tensor-core path size its launches
    quarts, segs = {}, {}
    for cls, q in raw.items():
        qq, seg, lcl = workloads.group_by_class(basis, q)
        quarts[cls], segs[cls] = qq, (seg, lcl)
    dent = deck.density(basis, seed=args.seed)
    flops = {cls: workloads.quartet_flops(basis, q, *cls) for cls, q in quarts.items()}
    cflops = {cls: workloads.contraction_flops(basis, q, *cls) for cls, q in quarts.items()}
    fb = berthagpu.FockBuilder(basis)
    n = fb.ndim
    # complex matrices as interleaved doubles; the column-major (n x n) array
    # is the row-major transpose, which torch holds as [n, 2n]
    dent_rows = np.ascontiguousarray(dent.T).view(np.float64).reshape(n, 2 * n)
    D = torch.from_numpy(dent_rows).to(dev)
    GD = torch.zeros(n, 2 * n, dtype=torch.float64, device=dev)
    GX = torch.zeros_like(GD)
    dq = {cls: torch.from_numpy(q).to(dev) for cls, q in quarts.items()}
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream

    def step(events=None):
        launches = 0
        for k, (cls, q) in enumerate(dq.items()):
            if events is not None:
                events[k][0].record(stream)
            seg, lcl = segs[cls]
            fb.quartets_segments(q.data_ptr(), seg, lcl, cls[0], cls[1], D.data_ptr(),
                                 GD.data_ptr(), GX.data_ptr(), n, sp)
            launches += fb.launches()
            if events is not None:
                events[k][1].record(stream)
        return launches

    def matrices():
        gd = GD.cpu().numpy().view(np.complex128).reshape(n, n).T
        gx = GX.cpu().numpy().view(np.complex128).reshape(n, n).T
        return gd, gx

    def energy_terms():
        # one clean step; J/K as matrices
        GD.zero_()
        GX.zero_()
        step()
        torch.cuda.synchronize()
        return matrices()

    def timed(prec):
        fb.set_precision(prec)
        for _ in range(args.warmup):
            flush.zero_()
            step()
        torch.cuda.synchronize()
        ev = [[[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in dq]
              for _ in range(args.steps)]
        launches = 0
        with ClockSampler(local) as clk:
            if world > 1:
                dist.barrier()
            torch.cuda.synchronize()
            for s_ in range(args.steps):
                flush.zero_()
                launches += step(ev[s_])
            torch.cuda.synchronize()
            if world > 1:
                dist.barrier()
        kern_ms = np.array([[ev[s_][k][0].elapsed_time(ev[s_][k][1]) for k in range(len(dq))]
                            for s_ in range(args.steps)])
        return kern_ms, launches, clk.summary()

    peak64 = fp64_peak(torch)
    peak_tf32 = tf32_peak(torch)
    res = {}
    for prec in PATHS:
        if prec != args.precision:
            res[prec] = timed(prec)
    res[args.precision] = timed(args.precision)
    kern_ms, launches, clocks = res[args.precision]
    mats = {}
    for prec in PATHS:
        fb.set_precision(prec)
        mats[prec] = energy_terms()
    status = _lib.device_status()
    fb.set_precision(args.precision)
    gd64, gx64 = mats["fp64"]
    scale = max(np.abs(gd64).max(), np.abs(gx64).max())

    def e2(gd, gx):
        # 1/2 sum_ij D_ij G_ij, the reference's energy sum (ENRGIES)
        return (0.5 * np.sum(dent * gd).real, 0.5 * np.sum(dent * gx).real)

    ej64, ek64 = e2(gd64, gx64)
    accuracy = {"reference": "FP64 GPU path (itself within 1e-11 of the oracle in the tests)",
                "energy_j_eh": float(ej64), "energy_k_eh": float(ek64),
                "device_status": status}
    for prec in PATHS[1:]:
        gdm, gxm = mats[prec]
        ejm, ekm = e2(gdm, gxm)
        accuracy[prec] = {
            "j_max_abs": float(np.abs(gdm - gd64).max()),
            "k_max_abs": float(np.abs(gxm - gx64).max()),
            "rel_to_max_element": float(max(np.abs(gdm - gd64).max(),
                                            np.abs(gxm - gx64).max()) / scale),
            "energy_j_abs_eh": float(abs(ejm - ej64)),
            "energy_k_abs_eh": float(abs(ekm - ek64))}
    # a sample of the workload digested by the oracle: the FP64 path and
    # the headline path against the reference's arithmetic
    from oracle import oracle as orc
    O = orc.QuartetOracle(basis)
    osamp = {}
    for prec in ("fp64", args.precision):
        fb.set_precision(prec)
        err = 0.0
        sc = 0.0
        for cls, q in raw.items():
            sub = q[:1024]
            rd = np.zeros((n, n), complex, order="F")
            rx = np.zeros((n, n), complex, order="F")
            O.prepare(sub, *cls)
            O.digest(sub, *cls, dent, rd, rx, nthreads=os.cpu_count() or 1)
            dsub = torch.from_numpy(np.ascontiguousarray(sub)).to(dev)
            GD.zero_()
            GX.zero_()
            fb.quartets(dsub.data_ptr(), sub.shape[0], cls[0], cls[1], D.data_ptr(),
                        GD.data_ptr(), GX.data_ptr(), n, sp)
            torch.cuda.synchronize()
            gd, gx = matrices()
            err = max(err, float(np.abs(gd - rd).max()), float(np.abs(gx - rx).max()))
            sc = max(sc, float(np.abs(rd).max()), float(np.abs(rx).max()))
        osamp[prec] = {"max_abs": err, "rel_to_max_element": err / sc}
    O.close()
    accuracy["vs_oracle_4096_quartets"] = osamp
    fb.set_precision(args.precision)

    step_ms = float(kern_ms.sum(1).max() if args.steps else 0.0)
    step_ms_mean = float(kern_ms.sum(1).mean())
    ms_per_step = replicas.job_step_ms(step_ms_mean, dist if world > 1 else None, dev)
    value = replicas.job_throughput(args.quartets, world, ms_per_step)
    path_values = {p: {"value": args.quartets * world / (float(r[0].sum(1).mean()) * 1e-3),
                       "unit": UNIT, "ms_per_step": float(r[0].sum(1).mean())}
                   for p, r in res.items()}

    # quartets/s per angular class (l_a,l_b,l_c,l_d), all component classes
    # together, FP64 and the headline path: one launch per class segment
    per_ang = {}
    for prec in ("fp64", args.precision):
        fb.set_precision(prec)
        evs = []
        for cls, q in dq.items():
            seg, lcl = segs[cls]
            for i in range(len(seg) - 1):
                key = "".join(str(int(x)) for x in lcl[i])
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                fb.quartets_segments(q[int(seg[i]):].data_ptr(), seg[i:i + 2] - seg[i],
                                     lcl[i:i + 1], cls[0], cls[1], D.data_ptr(), GD.data_ptr(),
                                     GX.data_ptr(), n, sp)
                b.record(stream)
                evs.append((key, int(seg[i + 1] - seg[i]), a, b))
        torch.cuda.synchronize()
        for key, m, a, b in evs:
            e = per_ang.setdefault(key, {"quartets": 0})
            e["quartets"] += m
            e[prec + "_ms"] = e.get(prec + "_ms", 0.0) + a.elapsed_time(b)
    per_angular_class = {k: {"quartets": v["quartets"],
                             **{p + "_qps": v["quartets"] / (v[p + "_ms"] * 1e-3)
                                for p in ("fp64", args.precision)}}
                         for k, v in sorted(per_ang.items(), reverse=True)}
    fb.set_precision(args.precision)

    # end to end through the C ABI: host density and quartet lists in pinned
    # memory copied in, J/K copied back, every step
    hD = torch.from_numpy(dent_rows).pin_memory()
    hq = {cls: torch.from_numpy(q).pin_memory() for cls, q in quarts.items()}
    hGD = torch.empty(GD.shape, dtype=torch.float64).pin_memory()
    hGX = torch.empty(GX.shape, dtype=torch.float64).pin_memory()
    h2d = hD.numel() * 8 + sum(v.numel() * 4 for v in hq.values())
    d2h = 2 * hGD.numel() * 8
    e_ms = []
    for s_ in range(max(1, min(args.steps, 3))):
        flush.zero_()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        D.copy_(hD, non_blocking=True)
        for cls in dq:
            dq[cls].copy_(hq[cls], non_blocking=True)
        GD.zero_()
        GX.zero_()
        step()
        hGD.copy_(GD, non_blocking=True)
        hGX.copy_(GX, non_blocking=True)
        b.record(stream)
        b.synchronize()
        e_ms.append(a.elapsed_time(b))
    e2e_value = args.quartets / (float(np.mean(e_ms)) * 1e-3)

    # rooflines: the headline kernel (tensor pipe for tc32: 3 TF32 MMAs per
    # product of the dense contraction count; FP64 pipe otherwise) and the
    # FP64 kernel beside it
    tot_flops = sum(flops.values())
    tot_cflops = sum(cflops.values())
    kern_mean = kern_ms.mean(0)
    t_head = kern_mean.sum() * 1e-3
    t64 = res["fp64"][0].mean(0).sum() * 1e-3
    fp64_roof = {"bound": "fp64", "kernel": "k_quartet", "achieved": tot_flops / t64 / 1e12,
                 "peak": peak64, "unit": "TFLOP/s", "frac": tot_flops / t64 / 1e12 / peak64,
                 "peak_source": "cuBLAS DGEMM 4096^3 measured in this run"}
    if args.precision == "tc32":
        ach = 3.0 * tot_cflops / t_head / 1e12
        roofline = {"bound": "tensor", "kernel": "k_quartet_tc", "achieved": ach,
                    "peak": peak_tf32, "unit": "TFLOP/s", "frac": ach / peak_tf32,
                    "peak_source": "cuBLAS TF32 GEMM 8192^3 measured in this run "
                                   "(MEASURED_PEAKS.json has no TF32 entry)",
                    "flops_per_step": 3.0 * tot_cflops,
                    "traffic": TC_TRAFFIC_BYTES_PER_STEP,
                    "traffic_per": "step (all k_quartet_tc launches of one step, as achieved)",
                    "fp64_kernel": fp64_roof}
    else:
        roofline = dict(fp64_roof)
        roofline["traffic"] = read_traffic()
        roofline["flops_per_step"] = tot_flops

    line = None
    h2o = breit = scf = tlf = atoms = None
    if rank == 0 and not args.no_h2o:
        h2o = h2o_fock_build(torch, with_cpu=(world == 1))
        breit = h2o_breit_build(torch)
        scf = h2o_scf(torch)
        tlf = tlf_builds(torch)
        atoms = batched_atoms(torch)
    if rank == 0:
        cpu = None
        if world == 1:
            r, nq, t = cpu_rate(basis, raw, dent, args.cpu_seconds, os.cpu_count() or 1)
            cpu = {"value": r, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                   "sample": f"{nq} quartets (equal per class) of the same workload, {t:.1f} s, "
                             "C++ restatement of bertha-scf.f ERIFAST/CLMMTG"}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": DTYPE[args.precision],
            "data": "synthetic",
            "config": config(args),
            "quartets_per_step": args.quartets,
            "precision": args.precision,
            "step_ms_max": step_ms,
            "paths": path_values,
            "speedup_vs_fp64": {p: path_values[p]["value"] / path_values["fp64"]["value"]
                                for p in PATHS},
            "accuracy_vs_fp64": accuracy,
            "per_component_class_ms": {f"{'LS'[c[0]]}{'LS'[c[0]]}|{'LS'[c[1]]}{'LS'[c[1]]}":
                                       float(kern_mean[k]) for k, c in enumerate(dq)},
            "per_angular_class": per_angular_class,
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                    "d2h_bytes_per_step": int(d2h)},
            "gpu_launches": int(launches),
            "clocks": clocks,
            "fock_build_h2o": h2o,
            "breit_build_h2o": breit,
            "scf_h2o": scf,
            "fock_build_tlf": tlf,
            "batched_atoms": atoms,
        }
        print(json.dumps(line), flush=True)
    fb.close()
    if world > 1:
        dist.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        if int(os.environ.get("RANK", 0)) != 0:
            return
        run_reference(args)
        return
    run_gpu(args)


if __name__ == "__main__":
    main()

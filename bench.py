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
    p.add_argument("--no-h2o", action="store_true",
                   help="skip the other configurations (H2O builds and SCF, TlF builds, "
                        "batched atoms) reported beside the headline")
    p.add_argument("--precision", default="df32", choices=["fp64", "df32"],
                   help="precision of the headline value; the other is timed beside it")
    return p.parse_args()


def config(args, extra=None):
    c = {"workload": WORKLOAD, "quartets_per_step": args.quartets, "seed": args.seed,
         "pool": "32 centres x 4 l x 2 exponents (256 shells, NDIM 4096)",
         "l2": "flushed between timed steps (256 MiB write)",
         "parallelism": f"replicas x{args.gpus}"}
    if extra:
        c.update(extra)
    return c


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
    from berthagpu import deck, workloads
    basis = workloads.microbench_pool(seed=args.seed)
    quarts = workloads.microbench_quartets(basis, args.quartets, seed=args.seed)
    dent = deck.density(basis, seed=args.seed)
    cores = os.cpu_count() or 1
    rates = []
    per_step = max(2.0, min(args.cpu_seconds, 120.0 / max(1, args.steps + args.warmup)))
    for i in range(args.warmup + args.steps):
        r, nq, t = cpu_rate(basis, quarts, dent, per_step, cores)
        if i >= args.warmup:
            rates.append((r, nq, t))
    value = float(np.mean([r for r, _, _ in rates]))
    sample = (f"{rates[-1][1]} quartets per step (equal per component class) of the "
              f"{args.quartets}-quartet workload, {rates[-1][2]:.1f} s")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * args.quartets / value, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": config(args), "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": sample},
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
    for prec in ("fp64", "df32"):
        fb = berthagpu.FockBuilder(b)
        fb.set_precision(prec)
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
    out["split_energy_err_eh"] = float(max(abs(e["df32"][0] - e["fp64"][0]),
                                           abs(e["df32"][1] - e["fp64"][1])))
    if with_cpu:
        from oracle import oracle as orc
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
    out = {"molecule": "H2O", "ndim": b.ndim, "nocc": 10, "screen": 1e-12, "etol_eh": 1e-9}
    for prec in ("fp64", "df32"):
        scf = DHFSCF(b, nocc=10, precision=prec, screen=1e-12, torch=torch)
        r = scf.run(max_iter=60, etol=1e-9)
        scf.close()
        out[prec] = {k: r[k] for k in ("energy", "iterations", "converged", "wall_s", "fock_s",
                                       "linalg_s", "oneel_s")}
    out["energy_diff_split_vs_fp64_eh"] = abs(out["df32"]["energy"] - out["fp64"]["energy"])
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


def tlf_builds(torch):
    """The TlF Dirac-Coulomb-Breit configuration (R = 3.94 bohr on z, Tl
    28s24p16d12f and F 14s9p3d even-tempered, Schwarz 1e-12, DIATOM: real
    digestion): one stage-3 Coulomb build in FP64 and in the autotuned mixed
    mode, and the Breit build in FP64, on device arrays (seeded Hermitian
    density), each timed with CUDA events after a first call that builds
    the lists (and, for the mixed mode, tunes the kernel per class)."""
    import berthagpu
    from berthagpu import deck
    b = deck.tlf_basis()
    dent = deck.density(b, seed=1, real=True)
    n = b.ndim
    d_D = torch.from_numpy(np.ascontiguousarray(dent.T)).cuda()
    J, K, B = (torch.zeros((n, n), dtype=torch.complex128, device="cuda") for _ in range(3))
    out = {"ndim": n, "shells": len(b.shells()), "hmlt": "DHFB", "screen": 1e-12, "ilev": 3}
    for prec in ("fp64", "auto"):
        fb = berthagpu.FockBuilder(b)
        fb.set_precision(prec)
        fb.set_screening(1e-12)
        t0 = time.perf_counter()
        fb.clmfast_device(d_D.data_ptr(), J.data_ptr(), K.data_ptr(), 3, n)
        torch.cuda.synchronize()
        first = time.perf_counter() - t0
        t = _device_time(torch, lambda s: fb.clmfast_device(d_D.data_ptr(), J.data_ptr(),
                                                           K.data_ptr(), 3, n, s))
        r = {"first_call_s": first, "device_s": t,
             "energy_j_eh": float(0.5 * torch.sum(d_D * J).real),
             "energy_k_eh": float(0.5 * torch.sum(d_D * K).real)}
        if prec == "auto":
            r["auto"] = fb.auto_stats()
        else:
            fb.brtfast_device(d_D.data_ptr(), B.data_ptr(), 3, n)
            torch.cuda.synchronize()
            out["breit_fp64"] = {
                "device_s": _device_time(torch, lambda s: fb.brtfast_device(
                    d_D.data_ptr(), B.data_ptr(), 3, n, s)),
                "energy_bx_eh": float(0.5 * torch.sum(d_D * B).real)}
        fb.close()
        out["coulomb_" + prec] = r
    out["auto_vs_fp64_energy_abs_eh"] = max(
        abs(out["coulomb_auto"]["energy_j_eh"] - out["coulomb_fp64"]["energy_j_eh"]),
        abs(out["coulomb_auto"]["energy_k_eh"] - out["coulomb_fp64"]["energy_k_eh"]))
    out["dcb_fock_build_fp64_s"] = out["coulomb_fp64"]["device_s"] + out["breit_fp64"]["device_s"]
    # the precision's effect on a converged DCB total energy: the small TlF
    # case (same geometry, angular momenta and exponent range) from the
    # bare-nucleus start with maximum-overlap occupation from iteration 3,
    # FP64 and autotuned mixed precision
    from berthagpu.scf import DHFSCF
    bs = deck.tlf_small_basis()
    scf = {"case": "TlF, Tl 7s6p4d3f / F 4s3p1d, DHFB", "ndim": bs.ndim, "nocc": 90,
           "guess": "bare nucleus, maximum overlap from iteration 3", "etol_eh": 1e-8}
    for prec in ("fp64", "auto"):
        s = DHFSCF(bs, nocc=90, precision=prec, screen=1e-12, torch=torch)
        r = s.run(max_iter=120, etol=1e-8, mom=3)
        s.close()
        scf[prec] = {k: r[k] for k in ("energy", "iterations", "converged", "wall_s", "fock_s")}
    scf["energy_auto_vs_fp64_eh"] = abs(scf["auto"]["energy"] - scf["fp64"]["energy"])
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


def run_gpu(args):
    import torch
    import torch.distributed as dist

    import berthagpu
    from berthagpu import deck, replicas, workloads
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
    quarts = workloads.microbench_quartets(basis, args.quartets, seed=args.seed)
    dent = deck.density(basis, seed=args.seed)
    flops = {cls: workloads.quartet_flops(basis, q, *cls) for cls, q in quarts.items()}
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
            fb.quartets(q.data_ptr(), q.shape[0], cls[0], cls[1], D.data_ptr(),
                        GD.data_ptr(), GX.data_ptr(), n, sp)
            launches += fb.launches()
            if events is not None:
                events[k][1].record(stream)
        return launches

    def energy_terms():
        # one clean step; J/K contracted with the density (the two-electron
        # energy terms 1/2 Re tr(D J), 1/2 Re tr(D K), ENRGIES form)
        GD.zero_()
        GX.zero_()
        step()
        torch.cuda.synchronize()
        gd = GD.cpu().numpy().view(np.complex128).reshape(n, n).T
        gx = GX.cpu().numpy().view(np.complex128).reshape(n, n).T
        return gd, gx

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
            for s in range(args.steps):
                flush.zero_()
                launches += step(ev[s])
            torch.cuda.synchronize()
            if world > 1:
                dist.barrier()
        kern_ms = np.array([[ev[s][k][0].elapsed_time(ev[s][k][1]) for k in range(len(dq))]
                            for s in range(args.steps)])
        return kern_ms, launches, clk.summary()

    peak64 = fp64_peak(torch)
    other = "fp64" if args.precision == "df32" else "df32"
    kern_other, _, _ = timed(other)
    kern_ms, launches, clocks = timed(args.precision)
    fb.set_precision("fp64")
    gd64, gx64 = energy_terms()
    fb.set_precision("df32")
    gdm, gxm = energy_terms()
    fb.set_precision(args.precision)
    scale = max(np.abs(gd64).max(), np.abs(gx64).max())

    def e2(gd, gx):
        # 1/2 sum_ij D_ij G_ij, the reference's energy sum (ENRGIES)
        return (0.5 * np.sum(dent * gd).real, 0.5 * np.sum(dent * gx).real)

    ej64, ek64 = e2(gd64, gx64)
    ejm, ekm = e2(gdm, gxm)
    accuracy = {"j_max_abs": float(np.abs(gdm - gd64).max()),
                "k_max_abs": float(np.abs(gxm - gx64).max()),
                "rel_to_max_element": float(max(np.abs(gdm - gd64).max(),
                                                np.abs(gxm - gx64).max()) / scale),
                "energy_j_abs_eh": float(abs(ejm - ej64)),
                "energy_k_abs_eh": float(abs(ekm - ek64)),
                "energy_j_eh": float(ej64), "energy_k_eh": float(ek64)}
    step_ms = float(kern_ms.sum(1).max() if args.steps else 0.0)
    step_ms_mean = float(kern_ms.sum(1).mean())
    ms_per_step = replicas.job_step_ms(step_ms_mean, dist if world > 1 else None, dev)
    value = replicas.job_throughput(args.quartets, world, ms_per_step)
    other_value = args.quartets * world / (float(kern_other.sum(1).mean()) * 1e-3)

    # end to end through the C ABI: host density and quartet lists in pinned
    # memory copied in, J/K copied back, every step
    hD = torch.from_numpy(dent_rows).pin_memory()
    hq = {cls: torch.from_numpy(q).pin_memory() for cls, q in quarts.items()}
    hGD = torch.empty(GD.shape, dtype=torch.float64).pin_memory()
    hGX = torch.empty(GX.shape, dtype=torch.float64).pin_memory()
    h2d = hD.numel() * 8 + sum(v.numel() * 4 for v in hq.values())
    d2h = 2 * hGD.numel() * 8
    e_ms = []
    for s in range(max(1, min(args.steps, 3))):
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

    tot_flops = sum(flops.values())
    kern_mean = kern_ms.mean(0)
    achieved = tot_flops / (kern_mean.sum() * 1e-3) / 1e12
    kern64 = kern_ms if args.precision == "fp64" else kern_other
    achieved64 = tot_flops / (kern64.mean(0).sum() * 1e-3) / 1e12
    per_class = {f"{'LS'[c[0]]}{'LS'[c[0]]}|{'LS'[c[1]]}{'LS'[c[1]]}":
                 {"ms": float(kern_mean[k]), "quartets_per_s": float(quarts[c].shape[0] / (kern_mean[k] * 1e-3)),
                  "tflops": float(flops[c] / (kern_mean[k] * 1e-3) / 1e12)}
                 for k, c in enumerate(dq)}
    traffic = read_traffic()

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
            r, nq, t = cpu_rate(basis, quarts, dent, args.cpu_seconds, os.cpu_count() or 1)
            cpu = {"value": r, "unit": UNIT, "cores": os.cpu_count() or 1, "kind": "port",
                   "sample": f"{nq} quartets (equal per class) of the same workload, {t:.1f} s, "
                             "C++ restatement of bertha-scf.f ERIFAST/CLMMTG"}
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_per_step,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": ("f64" if args.precision == "fp64" else
                      "f32x2 double-float contractions; f64 Boys, R, J/K sums"),
            "data": "synthetic",
            "config": config(args, {"precision": args.precision, "per_class": per_class,
                                    "step_ms_max": step_ms}),
            "fp64_path": {"value": value if args.precision == "fp64" else other_value,
                          "unit": UNIT},
            "split_precision_path": {"value": value if args.precision == "df32" else other_value,
                                     "unit": UNIT},
            "speedup_split_vs_fp64": (value / other_value if args.precision == "df32"
                                      else other_value / value),
            "accuracy_split_vs_fp64": accuracy,
            "roofline": {"bound": "fp64", "kernel": "k_quartet (FP64 path)",
                         "achieved": achieved64,
                         "peak": peak64, "unit": "TFLOP/s", "frac": achieved64 / peak64,
                         "peak_source": "cuBLAS DGEMM 4096^3 measured in this run "
                                        "(MEASURED_PEAKS.json has no FP64 entry)",
                         "traffic": traffic,
                         "flops_per_step": tot_flops,
                         "split_path_effective_tflops": achieved},
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

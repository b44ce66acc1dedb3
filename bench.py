#!/usr/bin/env python3
"""Benchmark: ms per SCF grid Fock build on one GB300, mixed vs FP64.

Workload (the headline configuration): benzene D6h (C-C 2.640, C-H 2.040
bohr), 6-31G (66 basis functions), 75 radial x 302 Lebedev points per atom,
lmax 8: 271,800 grid points.  A step is one grid Fock build at a fixed density
matrix P: rho on the grid, density correction, Slater+VWN point kernel,
Becke-Poisson Hartree potential, J and XC.  P is the density of the reference
program's own SCF (tests/golden/ref_benzene_p631_75x302.npz), the same in both
arms.

  value     ms per build in mixed precision, P already in HBM, device-timed with
            CUDA events on the library's stream, L2 flushed before every step
  e2e       the same metric through dftg_fock_build (host buffers: P copied in,
            J, XC, E_xc, N copied out, all inside the timed region)
  fp64      the same build with every step in FP64 (the metric's comparison)
  accuracy  |dE_tot| between mixed and FP64 SCF energies at convergence,
            max|dJ|, max|dXC| at the converged P, and both builds against the
            reference program's own J, XC, E_xc and E_J at the fixed P
  roofline  dominant kernel of the mixed build: its algorithmic bytes (the
            per-point operand bytes of the contraction or density formula)
            over its measured duration, against the measured HBM copy
            bandwidth; the layout bytes it actually streams as a second field
  adjoint   alkanes CnH2n+2 / 6-31G / 50 x 194: mixed forward and backward
            (dE/dP, forces) times and force errors (outside the headline)
  batched   64 jittered small molecules: one persistent launch per step over
            all molecules, and one CUDA graph of per-molecule branches, vs
            per-molecule builds, with the batch autotuner (outside the headline)
  synthetic 2M points x 512 primitives: rho, LDA and XC in FP64 and mixed
            (outside the headline)

--impl reference times the reference algorithm on the host cores for the same
workload: every step one whole, unsampled build by the C port of the
reference's path under oracle/ (OpenMP on all cores).  The reference program
itself builds only where its sources are (oracle/_ref); its outputs pin the
port to 1e-12 (tests/test_reference_pin.py).
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "ms per SCF grid Fock build, mixed vs FP64 on one GB300 at |\u0394E_tot|\u22641e-6 Ha"
WORKLOAD = {"workload": "benzene/6-31G grid Fock build", "molecule": "C6H6 D6h", "basis": "6-31G", "nbf": 66,
            "radial_points": 75, "lebedev_points": 302, "lmax": 8, "grid_points": 271800,
            "density_matrix": "the reference program's SCF density (30 x 110 grid, |dE| <= 1e-9)",
            "l2": "GPU arm: flushed (256 MB write) before every step"}
DTYPE = "fp16 fixed-point slices (3, density) and bf16 slices (3, contraction) + fp32 accumulate, fp64 reductions"
REF_FIXTURE = os.path.join(ROOT, "tests", "golden", "ref_benzene_p631_75x302.npz")


def _fixed_density():
    """The workload's fixed density matrix (the reference program's SCF P) and
    the reference program's outputs at it."""
    return dict(np.load(REF_FIXTURE))

# kernels launched per phase of one mixed-precision build (dftg_fock_build_device):
# density = P slicing with the correction factor + the tensor-core density with
# the LDA point kernel; multipole = rho_lm, Poisson and splines; vcross = the
# pair evaluation + the own-cell / total potential with E_J
KERNELS_PER_PHASE = {"density_slices": 1, "density": 1, "charge": 1, "lda": 1, "multipole": 1, "rholm": 1,
                     "poisson": 1, "vown": 1, "splines": 1, "vcross_bins": 1, "vcross": 1, "hartree_energy": 1,
                     "contract_bounds": 1, "contract": 1, "contract_reduce": 1}


def _env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def _peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), float(d["bf16_tflops"]), "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.proc = None
        self.path = None

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.2)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        rows = []
        try:
            with open(self.path) as f:
                for line in f:
                    p = [x.strip() for x in line.split(",")]
                    if len(p) >= 9:
                        rows.append(p)
        except Exception:
            pass
        finally:
            try:
                os.unlink(self.path)
            except Exception:
                pass
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if "Active" in r[5 + i] and "Not" not in r[5 + i]})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def max_over_ranks(values, device="cpu"):
    """Element-wise maximum of a list of floats over all ranks of the default group."""
    import torch
    t = torch.tensor(values, dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return [float(x) for x in t.tolist()]


def _benzene_mol():
    from dftcxx_gb300.molecule import Molecule, benzene
    Z, xyz = benzene()
    return Molecule(Z, xyz, "p631", "benzene")


def run_reference(args, rank):
    """Reference algorithm (C port, oracle/) on all host cores: every step one
    whole, unsampled build at the workload's fixed P."""
    if rank != 0:
        return None
    from oracle import oracle
    oracle.build()
    mol = _benzene_mol()
    g = oracle.OracleGrid(mol, 75, 11, 8)
    P = _fixed_density()["P"]
    cores = oracle.lib().orc_num_threads()

    def step():
        t0 = time.perf_counter()
        g.set_density(P)
        g.correct_densities()
        g.hartree()
        g.xc()
        return (time.perf_counter() - t0) * 1e3

    for _ in range(args.warmup):
        step()
    times = [step() for _ in range(args.steps)]
    ms = float(np.mean(times))
    sample = ("benzene/6-31G/75x302 grid Fock build, whole (every point, every phase), "
              "one build per step at the reference program's SCF density")
    return {"metric": METRIC, "value": ms, "unit": "ms", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic geometry (no dataset)",
            "config": dict(WORKLOAD), "impl": "reference", "parallelism": "host OpenMP, %d threads" % cores,
            "cpu_baseline": {"value": ms, "unit": "ms", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": ms, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def _scf(grid, mol, S, H, enuc, precision, tol=1e-8, max_iter=200):
    """Reference SCF iteration (dft.cpp:84-142) on one context."""
    grid.set_precision(precision)
    lam, U = np.linalg.eigh(S)
    X = U @ np.diag(1.0 / np.sqrt(lam))
    nocc = mol.nelec // 2
    n = mol.nbf
    J = np.zeros((n, n))
    XC = np.zeros((n, n))
    P = None

    def dens(P):
        _, Cp = np.linalg.eigh(X.T @ (H + 2 * J + XC) @ X)
        C = X @ Cp
        Pn = C[:, :nocc] @ C[:, :nocc].T
        return Pn if P is None else 0.5 * Pn + 0.5 * P

    P = dens(P)
    grid.set_density(P)
    grid.correct_densities()
    J = grid.calculate_hartree_potential()
    exc = 0.0
    E = 2 * np.trace(P @ H) + 2 * np.trace(P @ J) + enuc + exc
    old, it = E, 0
    while True:
        it += 1
        P = dens(P)
        r = grid.fock_build(P)
        J, XC, exc = r["J"], r["XC"], r["Exc"]
        E = 2 * np.trace(P @ H) + r["EJ"] + enuc + exc     # E_J = 2 tr(P J) summed on the grid
        if (abs(E - old) < tol and it >= 3) or it >= max_iter:
            return E, P, it
        old = E


def _device_scf(mol, dev, precision, tol=1e-8, max_iter=200):
    """The reference SCF (dft.cpp:84-142) run by the device driver: one CUDA
    graph launch for the whole loop; wall times around set-up and run."""
    import torch
    from dftcxx_gb300.grid import DeviceSCF
    t0 = time.perf_counter()
    ds = DeviceSCF(mol, 75, 11, 8, precision=precision, device=dev, tol=tol, max_iter=max_iter)
    t1 = time.perf_counter()
    E = ds.run()
    torch.cuda.synchronize(dev)
    t2 = time.perf_counter()
    out = {"E_Ha": E, "iterations": ds.iterations, "setup_ms": 1e3 * (t1 - t0), "run_ms": 1e3 * (t2 - t1),
           "ms_per_iteration": 1e3 * (t2 - t1) / max(1, ds.iterations),
           "loop": {1: "one conditional-graph launch", 2: "one graph launch per iteration"}[ds.diagnostics()["mode"]],
           "P": ds.P}
    ds.close()
    return out


def run_ours(args, rank, world):
    import torch
    from dftcxx_gb300 import build as b
    from dftcxx_gb300 import _lib
    from dftcxx_gb300.grid import MolecularGrid
    b.build()
    L = _lib.load()
    dev = _env_int("LOCAL_RANK", 0)
    torch.cuda.set_device(dev)
    mol = _benzene_mol()
    grid = MolecularGrid(mol, 75, 11, 8, precision="mixed", device=dev)
    S, T, V = grid.one_electron()
    H = T + V
    enuc = grid.nuclear_repulsion()

    # accuracy: converged SCF in both precisions on the device driver, and the
    # host-driven loop (numpy eigen-solves) for comparison (outside the timed region)
    t0 = time.perf_counter()
    scf_dev = {p: _device_scf(mol, dev, p) for p in ("fp64", "mixed")}
    E64, P64, it64 = scf_dev["fp64"]["E_Ha"], scf_dev["fp64"].pop("P"), scf_dev["fp64"]["iterations"]
    Emx, Pmx, itmx = scf_dev["mixed"]["E_Ha"], scf_dev["mixed"].pop("P"), scf_dev["mixed"]["iterations"]
    th = time.perf_counter()
    Eh, _, ith = _scf(grid, mol, S, H, enuc, "mixed")
    th = time.perf_counter() - th
    scf_info = {"device": scf_dev, "host_loop_mixed": {"E_Ha": Eh, "iterations": ith,
                                                       "ms_per_iteration": 1e3 * th / max(1, ith)},
                "dE_device_vs_host_loop_mixed_Ha": abs(Emx - Eh)}
    scf_s = time.perf_counter() - t0
    grid.set_precision("fp64")
    r64 = grid.fock_build(P64)
    grid.set_precision("mixed")
    rmx = grid.fock_build(P64)
    dE_fixedP = abs(rmx["EJ"] - r64["EJ"] + rmx["Exc"] - r64["Exc"])
    dE_Jmatrix = abs(2 * np.trace(P64 @ (rmx["J"] - r64["J"])))
    # error budget: each step alone in its mixed form, at the converged FP64 density
    ablation = {}
    for name, bit in grid.MIX_BITS.items():
        grid.set_precision_mask(bit)
        rb = grid.fock_build(P64)
        ablation[name] = {"dE_tot_Ha": float(rb["EJ"] - r64["EJ"] + rb["Exc"] - r64["Exc"]),
                          "dE_2trPdJ_Ha": float(2 * np.trace(P64 @ (rb["J"] - r64["J"]))),
                          "max_dJ": float(np.abs(rb["J"] - r64["J"]).max()),
                          "max_dXC": float(np.abs(rb["XC"] - r64["XC"]).max())}
    accuracy = {"dE_tot_scf_Ha": abs(E64 - Emx), "E_tot_fp64_Ha": E64, "E_tot_mixed_Ha": Emx,
                "scf_iterations": [it64, itmx], "dE_tot_fixed_P_Ha": dE_fixedP,
                "max_dJ": float(np.abs(rmx["J"] - r64["J"]).max()),
                "max_dXC": float(np.abs(rmx["XC"] - r64["XC"]).max()),
                "dExc_Ha": abs(rmx["Exc"] - r64["Exc"]), "dE_2trPdJ_Ha": dE_Jmatrix,
                "dE_J_grid_fp64_vs_2trPJ_Ha": abs(r64["EJ"] - 2 * np.trace(P64 @ r64["J"])),
                "per_step": ablation}
    # both builds against the reference program's own outputs at the fixed P
    fx = _fixed_density()
    Pfix = fx["P"]
    vs_ref = {}
    for prec in ("fp64", "mixed"):
        grid.set_precision(prec)
        rr = grid.fock_build(Pfix)
        vs_ref[prec] = {"dE_tot_Ha": float((rr["EJ"] - fx["scalars"][1]) + (rr["Exc"] - fx["scalars"][0])),
                        "dE_xc_Ha": float(rr["Exc"] - fx["scalars"][0]),
                        "dE_J_Ha": float(rr["EJ"] - fx["scalars"][1]),
                        "max_dJ": float(np.abs(rr["J"] - fx["J"]).max()),
                        "max_dXC": float(np.abs(rr["XC"] - fx["XC"]).max())}
    accuracy["vs_reference_program_fixed_P"] = vs_ref
    grid.set_precision("mixed")

    stream = torch.cuda.Stream(device=dev)
    grid.set_stream(stream.cuda_stream)
    nn = mol.nbf * mol.nbf
    dP = torch.from_numpy(np.asfortranarray(Pfix).ravel(order="F").copy()).to(f"cuda:{dev}")
    dJ = torch.zeros(nn, dtype=torch.float64, device=f"cuda:{dev}")
    dXC = torch.zeros_like(dJ)
    dS = torch.zeros(2, dtype=torch.float64, device=f"cuda:{dev}")
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{dev}")   # > 129 MB L2

    def dev_step():
        rc = L.dftg_fock_build_device(grid.handle, ctypes.c_void_p(dP.data_ptr()), ctypes.c_void_p(dJ.data_ptr()),
                                      ctypes.c_void_p(dXC.data_ptr()), ctypes.c_void_p(dS.data_ptr()))
        _lib.check(rc)

    def timed(precision, steps, warmup):
        grid.set_precision(precision)
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                flush.zero_()
                dev_step()
            torch.cuda.synchronize(dev)
            if world > 1:
                torch.distributed.barrier()
            evs = []
            torch.cuda.nvtx.range_push("timed_" + precision)
            for _ in range(steps):
                flush.zero_()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                dev_step()
                e1.record(stream)
                evs.append((e0, e1))
            torch.cuda.nvtx.range_pop()
            torch.cuda.synchronize(dev)
        return [a.elapsed_time(b) for a, b in evs]

    def profile(precision, reps=5):
        grid.set_precision(precision)
        acc = {}
        ms = (ctypes.c_double * 24)()
        names = (ctypes.c_char_p * 24)()
        n = ctypes.c_int()
        for _ in range(reps):
            with torch.cuda.stream(stream):
                flush.zero_()
            _lib.check(L.dftg_fock_build_profile(grid.handle, ctypes.c_void_p(dP.data_ptr()), ms, names, 24,
                                                 ctypes.byref(n)))
            for i in range(n.value):
                k = names[i].decode()
                acc.setdefault(k, []).append(ms[i])
        return {k: float(np.mean(v)) for k, v in acc.items()}

    with ClockSampler(dev) as clk:
        t_mx = timed("mixed", args.steps, args.warmup)
        t_64 = timed("fp64", max(3, min(args.steps, 10)), 3)
    clocks = clk.summary()
    ms_mx = float(np.mean(t_mx))
    ms_64 = float(np.mean(t_64))
    prof_mx = profile("mixed")
    prof_64 = profile("fp64")

    # end to end through the public host-buffer call
    grid.set_precision("mixed")
    grid.set_stream(0)
    hP = torch.from_numpy(np.asfortranarray(Pfix).ravel(order="F").copy()).pin_memory()
    hJ = torch.zeros(nn, dtype=torch.float64).pin_memory()
    hXC = torch.zeros(nn, dtype=torch.float64).pin_memory()
    e_, n_ = ctypes.c_double(), ctypes.c_double()
    dp = ctypes.POINTER(ctypes.c_double)

    def e2e_step():
        _lib.check(L.dftg_fock_build(grid.handle, ctypes.cast(hP.data_ptr(), dp), ctypes.cast(hJ.data_ptr(), dp),
                                     ctypes.cast(hXC.data_ptr(), dp), ctypes.byref(e_), ctypes.byref(n_)))

    for _ in range(args.warmup):
        flush.zero_()
        torch.cuda.synchronize(dev)
        e2e_step()
    e2e = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        e2e_step()
        e2e.append((time.perf_counter() - t0) * 1e3)
    ms_e2e = float(np.mean(e2e))

    # max over ranks
    if world > 1:
        ms_mx, ms_e2e, ms_64 = max_over_ranks([ms_mx, ms_e2e, ms_64], f"cuda:{dev}")

    # roofline of the dominant mixed-precision kernel: its algorithmic bytes per
    # launch (the operand bytes of the formula, 6 bytes per amplitude: three
    # BF16 planes) over the per-phase CUDA-event time of that kernel; the
    # layout bytes it actually streams (padded rows and tiles, a fourth plane
    # for the density) as a second figure; DRAM traffic per launch from the
    # committed ncu summary
    hbm, _, peak_src = _peaks()
    npts, nbf = grid.grid_size, mol.nbf
    npad = (npts + 127) // 128 * 128
    kp, ar = (nbf + 15) // 16 * 16, (nbf + 7) // 8 * 8
    npairs = npts * (mol.natoms - 1)
    alg_bytes = {
        # rho = 2 phi^T P phi: Npts nbf amplitudes in, rho out, P in
        "density": 6 * npts * nbf + 8 * npts + 8 * nbf * nbf,
        # V_xc and J in one pass: Npts nbf amplitudes, two point coefficients
        "contract": 6 * npts * nbf + 16 * npts,
        # per pair: direction and 1/r (16 B), offset and bin (8 B) in, contribution (8 B) out
        "vcross_bins": 32 * npairs,
        # per point: pair places (4 B per atom), pair contributions (8 B per other
        # atom), w, rho, 1/r in; V, cj (FP64) and cj (FP32) out
        "vcross": npts * (12 * mol.natoms + 36),
        "lda": npts * (8 + 8 + 8) + npts * (8 + 4),
    }
    layout_bytes = {
        "density": 4 * npad * kp * 2 + 8 * npad,
        "contract": 3 * npad * ar * 2 + 2 * 4 * npad,
    }
    dom = max(prof_mx, key=lambda k: prof_mx[k])
    dom_ms = prof_mx[dom]
    traffic = None
    try:
        with open(os.path.join(ROOT, "profiles", "roofline_traffic.json")) as f:
            traffic = json.load(f).get(dom)
    except Exception:
        traffic = None
    roof = {"kernel": dom, "bound": "hbm", "unit": "GB/s", "peak": hbm, "peak_source": peak_src,
            "traffic": traffic}
    if dom in alg_bytes:
        ach = alg_bytes[dom] / (dom_ms * 1e-3) / 1e9
        roof.update(achieved=ach, frac=ach / hbm, bytes_per_launch=alg_bytes[dom], ms_per_launch=dom_ms)
        if dom in layout_bytes:
            roof["layout_bytes_per_launch"] = layout_bytes[dom]
            roof["layout_GBps"] = layout_bytes[dom] / (dom_ms * 1e-3) / 1e9
        if traffic:
            roof["traffic_over_alg_bytes"] = traffic / alg_bytes[dom]
    else:
        roof.update(achieved=None, frac=None)
    launches_per_step = sum(KERNELS_PER_PHASE.get(k, 1) for k in prof_mx)

    # CPU baseline: reference algorithm on the host cores, bounded sample
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        ref_args = argparse.Namespace(**vars(args))
        ref_args.steps, ref_args.warmup = 2, 0
        r = run_reference(ref_args, 0)
        cpu = r["cpu_baseline"]
        cpu["sample"] = "2 whole builds (" + cpu["sample"] + ")"

    adjoint = batched = synthetic = None
    if rank == 0 and world == 1:
        if not args.no_adjoint:
            adjoint = run_adjoint(dev)
        if not args.no_batched:
            batched = run_batched(dev)
        if not args.no_synthetic:
            synthetic = run_synthetic(dev)

    return {"metric": METRIC, "value": ms_mx, "unit": "ms",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_mx,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": DTYPE,
            "data": "synthetic geometry (no dataset)",
            "config": dict(WORKLOAD), "parallelism": "replicas" if world > 1 else "single GPU",
            "fp64_ms_per_step": ms_64, "speedup_vs_fp64": ms_64 / ms_mx, "accuracy": accuracy,
            "phases_ms_mixed": prof_mx, "phases_ms_fp64": prof_64,
            "e2e": {"value": ms_e2e, "unit": "ms", "h2d_bytes_per_step": 8 * nn,
                    "d2h_bytes_per_step": 2 * 8 * nn + 2 * 8},
            "roofline": roof, "cpu_baseline": cpu, "clocks": clocks,
            "gpu_launches": launches_per_step * args.steps,
            "scf_seconds_outside_timing": scf_s,
            "scf": scf_info, "adjoint": adjoint, "batched": batched, "synthetic": synthetic}


def _guess_density(grid, mol):
    """Half density matrix of the lowest core-Hamiltonian orbitals (the SCF
    driver's first density, dft.cpp:216-226, 300-366)."""
    S, T, V = grid.one_electron()
    lam, U = np.linalg.eigh(S)
    X = U / np.sqrt(lam)
    _, Cp = np.linalg.eigh(X.T @ (T + V) @ X)
    C = (X @ Cp)[:, :mol.nelec // 2]
    return C @ C.T


def _event_ms(fn, reps, stream):
    import torch
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / reps


def run_adjoint(dev, ns=(2, 4, 6, 8, 10), reps=5, h=1e-4):
    """Adjoint workload: staggered CnH2n+2 / 6-31G / 50 x 194 at the
    core-Hamiltonian density.  Per molecule: device time of the mixed forward
    build and of the backward (dE/dP and dE/dR), the FP64 backward, and the
    largest force difference between the mixed and the FP64 backward; for the
    smallest and the largest chain, central differences (h = 1e-4 bohr) of the
    FP64 forward on the largest force component."""
    import torch
    from dftcxx_gb300 import _lib
    from dftcxx_gb300.grid import MolecularGrid
    from dftcxx_gb300.molecule import Molecule, alkane
    L = _lib.load()
    stream = torch.cuda.Stream(device=dev)
    rows = []
    for n in ns:
        Z, xyz = alkane(n)
        mol = Molecule(Z, xyz, "p631")
        g = MolecularGrid(mol, 50, 10, 8, precision="fp64", device=dev)
        P = _guess_density(g, mol)
        g.fock_build(P)
        _, dR64 = g.backward()
        g.set_stream(stream.cuda_stream)
        nn = mol.nbf * mol.nbf
        dP = torch.from_numpy(np.asfortranarray(P).ravel(order="F").copy()).to(f"cuda:{dev}")
        bufs = torch.zeros(3 * nn + 3 + 3 * mol.natoms, dtype=torch.float64, device=f"cuda:{dev}")
        J, XC, sc = bufs[:nn], bufs[nn:2 * nn], bufs[2 * nn:2 * nn + 3]
        gP, gR = bufs[2 * nn + 3:3 * nn + 3], bufs[3 * nn + 3:]
        vp = lambda t: ctypes.c_void_p(t.data_ptr())

        def fwd():
            _lib.check(L.dftg_fock_build_device(g.handle, vp(dP), vp(J), vp(XC), vp(sc)))

        def bwd():
            _lib.check(L.dftg_backward_device(g.handle, 1.0, 1.0, vp(gP), vp(gR)))

        with torch.cuda.stream(stream):
            fwd(); bwd()
            bw64 = _event_ms(bwd, 2, stream)
            fw64 = _event_ms(fwd, 2, stream)
            g.set_precision("mixed")
            for _ in range(3):
                fwd(); bwd()
            fw = _event_ms(fwd, reps, stream)
            bw = _event_ms(bwd, reps, stream)
            fwd(); bwd()
            torch.cuda.synchronize(dev)
        dRm = gR.cpu().numpy().reshape(-1, 3)
        row = {"n": n, "natoms": mol.natoms, "nbf": mol.nbf, "grid_points": g.grid_size,
               "mixed_forward_ms": fw, "mixed_backward_ms": bw, "fp64_forward_ms": fw64, "fp64_backward_ms": bw64,
               "max_force_diff_mixed_vs_fp64_Ha_bohr": float(np.abs(dRm - dR64).max()),
               "max_force_Ha_bohr": float(np.abs(dR64).max())}
        if n in (ns[0], ns[-1]):
            a, d = np.unravel_index(np.abs(dR64).argmax(), dR64.shape)
            es = []
            for sgn in (1, -1):
                dx = np.zeros((mol.natoms, 3))
                dx[a, d] = sgn * h
                gd = MolecularGrid(mol.displaced(dx), 50, 10, 8, precision="fp64", device=dev)
                r = gd.fock_build(P)
                es.append(r["Exc"] + r["EJ"])
                gd.close()
            fd = (es[0] - es[1]) / (2 * h)
            row["fd_check"] = {"atom": int(a), "axis": int(d), "fd_fp64_forward": fd,
                               "err_fp64_backward": float(dR64[a, d] - fd), "err_mixed_backward": float(dRm[a, d] - fd)}
        rows.append(row)
        g.close()
    return {"workload": "staggered CnH2n+2 / 6-31G / 50 x 194 / lmax 8, core-Hamiltonian density",
            "gradient": "dE/dR of E_xc + E_J at fixed P (grid part of the nuclear forces) and dE/dP",
            "molecules": rows}


def run_batched(dev, nmol=64, reps=10, seed=20261204):
    """Batched workload: nmol geometries drawn in turn from H2, LiH, H2O, NH3,
    CH4, N2, CO, C2H6, C6H6, every nucleus displaced by N(0, 0.05 bohr),
    STO-3G and 6-31G alternating by round, 50 x 194 grid, each at its own
    core-Hamiltonian density.  Throughput in grid builds (SCF iterations) per
    second: the per-molecule FP64 build, the per-molecule mixed build, and the
    whole batch as persistent launches (one per step) and as one graph of
    per-molecule branches, before and after the batch autotuner."""
    import torch
    from dftcxx_gb300 import _lib
    from dftcxx_gb300.grid import MolecularGrid, Batch
    from dftcxx_gb300.molecule import Molecule, small_molecule
    L = _lib.load()
    names = ["H2", "LiH", "H2O", "NH3", "CH4", "N2", "CO", "C2H6", "C6H6"]
    rng = np.random.default_rng(seed)
    grids, dPs, outs = [], [], []
    natoms = nbfs = npts = 0
    cross_evals = 0
    t0 = time.perf_counter()
    for i in range(nmol):
        name = names[i % len(names)]
        basis = "sto3g" if (i // len(names)) % 2 == 0 else "p631"
        Z, xyz = small_molecule(name)
        xyz = np.asarray(xyz, dtype=float) + rng.normal(0.0, 0.05, size=(len(Z), 3))
        mol = Molecule(Z, xyz, basis)
        g = MolecularGrid(mol, 50, 10, 8, precision="fp64", device=dev)
        P = _guess_density(g, mol)
        nn = mol.nbf * mol.nbf
        grids.append(g)
        dPs.append(torch.from_numpy(np.asfortranarray(P).ravel(order="F").copy()).to(f"cuda:{dev}"))
        outs.append(torch.zeros(2 * nn + 3, dtype=torch.float64, device=f"cuda:{dev}"))
        natoms += mol.natoms
        nbfs += mol.nbf
        npts += g.grid_size
        cross_evals += g.grid_size * (mol.natoms - 1) * 81
    setup_s = time.perf_counter() - t0
    vp = lambda t: ctypes.c_void_p(t.data_ptr())
    # every leg is timed with events on this stream: the sequential builds run
    # on it, and the batch graph is launched on it (its branches fork from it
    # and join back into it)
    stream = torch.cuda.Stream(device=dev)

    def sequential():
        for g, P, o in zip(grids, dPs, outs):
            nn = g.nbf * g.nbf
            _lib.check(L.dftg_fock_build_device(g.handle, vp(P), vp(o[:nn]), vp(o[nn:2 * nn]), vp(o[2 * nn:])))

    torch.cuda.synchronize(dev)
    for g in grids:
        g.set_stream(stream.cuda_stream)
    sequential(); sequential()
    seq64 = _event_ms(sequential, 3, stream)
    for g in grids:
        g.set_precision("mixed")
    sequential(); sequential()
    seqmx = _event_ms(sequential, reps, stream)
    torch.cuda.synchronize(dev)
    for g in grids:   # every context back on its own stream: the graph's branches run concurrently
        g.set_stream(0)
    b = Batch(grids, mode="graph")
    Js = [o[:g.nbf * g.nbf] for g, o in zip(grids, outs)]
    XCs = [o[g.nbf * g.nbf:2 * g.nbf * g.nbf] for g, o in zip(grids, outs)]
    Ss = [o[2 * g.nbf * g.nbf:] for g, o in zip(grids, outs)]
    run = lambda: b.build(dPs, Js, XCs, Ss, stream=stream.cuda_stream)
    # graph of branches, then the persistent launches, at the set-up launch shapes
    run(); run()
    bat_g = _event_ms(run, reps, stream)
    b.set_mode("persistent")
    run(); run()
    bat_p = _event_ms(run, reps, stream)
    b.status()
    persistent = b.persistent_active()
    # each form autotuned (the persistent form last, so its shapes stay)
    b.set_mode("graph")
    run()
    tune_g = b.autotune(reps=5)
    run(); run()
    bat_gt = _event_ms(run, reps, stream)
    b.set_mode("persistent")
    run()
    t_tune = time.perf_counter()
    tune_p = b.autotune(reps=5)
    tune_s = time.perf_counter() - t_tune
    run(); run()
    bat_pt = _event_ms(run, reps, stream)
    # one replay with host wall-clock around it (synchronised on both sides)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    run()
    stream.synchronize()
    bat_wall = (time.perf_counter() - t0) * 1e3
    b.status()
    # the tuned persistent batch does the work: outputs zeroed, one replay, then
    # per-molecule builds of the same launch shapes must reproduce it bit for bit
    torch.cuda.synchronize(dev)
    for o in outs:
        o.zero_()
    torch.cuda.synchronize(dev)
    run()
    b.status()
    got = [o.clone() for o in outs]
    nonzero = all(bool(o.abs().max() > 0) for o in got)
    for g in grids:
        g.set_stream(stream.cuda_stream)
    sequential()
    torch.cuda.synchronize(dev)
    diff = max(float((a - b_).abs().max() / max(b_.abs().max(), 1e-300)) for a, b_ in zip(got, outs))
    shapes = sorted({g.launch_shape for g in grids})
    b.close()
    for g in grids:
        g.close()
    return {"workload": "%d geometries (H2 .. C6H6, N(0, 0.05 bohr) jitter), STO-3G / 6-31G, 50 x 194, lmax 8" % nmol,
            "atoms": natoms, "basis_functions": nbfs, "grid_points": npts,
            "fp64_per_molecule_builds_per_s": nmol / (seq64 * 1e-3),
            "mixed_per_molecule_builds_per_s": nmol / (seqmx * 1e-3),
            "mixed_batched_persistent_builds_per_s": nmol / (bat_pt * 1e-3),
            "mixed_batched_graph_builds_per_s": nmol / (bat_gt * 1e-3),
            "persistent_launches_ran": persistent,
            "launches_per_batch": {"persistent": "8 kernels + 1 memset", "graph": "8 kernels per molecule"},
            "ms_per_batch": {"fp64_sequential": seq64, "mixed_sequential": seqmx, "mixed_graph": bat_g,
                             "mixed_graph_autotuned": bat_gt, "mixed_persistent": bat_p,
                             "mixed_persistent_autotuned": bat_pt, "mixed_persistent_host_wall_one_replay": bat_wall,
                             "autotuner_best_graph": tune_g, "autotuner_best_persistent": tune_p},
            "cross_atom_evaluations": cross_evals,
            "max_rel_diff_batch_vs_single": diff, "batch_outputs_nonzero": nonzero,
            "autotuned_shapes": [list(s) for s in shapes], "autotune_s": tune_s, "setup_s": setup_s}


def run_synthetic(dev, npts=2_000_000, nbf=512, nocc=128, reps=3):
    """Synthetic contraction workload (seeded): 2M points uniform in a 20-bohr
    cube, weights log-uniform in [1e-4, 1], 512 single-primitive Cartesian
    s/p/d functions (exponents log-uniform in [0.1, 50], centres uniform in the
    cube), P = C C^T with C 512 x 128 ~ N(0, 0.1).  One step: rho = 2 phi^T P phi,
    LDA point kernel, XC = phi^T diag(w v_xc) phi (dftg_xc_build_device), FP64
    and mixed; the mixed error against FP64, the per-phase times, the BF16
    tensor rates of the density and contraction kernels, and the mixed step's
    rate over the operand bytes it streams."""
    import torch
    from dftcxx_gb300 import _lib
    from dftcxx_gb300.grid import PointGrid
    from dftcxx_gb300.molecule import synthetic_contraction
    L = _lib.load()
    t0 = time.perf_counter()
    pts, w, lmn, alpha, centres, P = synthetic_contraction(npts=npts, nbf=nbf, nocc=nocc)
    g = PointGrid(pts, w, centres, np.arange(nbf), lmn, np.ones(nbf, np.int32), alpha, np.ones(nbf),
                  precision="fp64", device=dev)
    setup_s = time.perf_counter() - t0
    stream = torch.cuda.Stream(device=dev)
    g.set_stream(stream.cuda_stream)
    nn = nbf * nbf
    dP = torch.from_numpy(np.asfortranarray(P).ravel(order="F").copy()).to(f"cuda:{dev}")
    XC = torch.zeros(nn, dtype=torch.float64, device=f"cuda:{dev}")
    sc = torch.zeros(2, dtype=torch.float64, device=f"cuda:{dev}")
    vp = lambda t: ctypes.c_void_p(t.data_ptr())

    def step():
        _lib.check(L.dftg_xc_build_device(g.handle, vp(dP), vp(XC), vp(sc)))

    with torch.cuda.stream(stream):
        step()
        ms64 = _event_ms(step, 1, stream)
        torch.cuda.synchronize(dev)
        xc64, s64 = XC.cpu().numpy().copy(), sc.cpu().numpy().copy()
        rho64 = g.get_densities()
        g.set_precision("mixed")
        step(); step()
        msmx = _event_ms(step, reps, stream)
        torch.cuda.synchronize(dev)
        xcm, sm = XC.cpu().numpy().copy(), sc.cpu().numpy().copy()
        rhom = g.get_densities()
        # per-phase CUDA-event times of the mixed step
        ms = (ctypes.c_double * 24)()
        names = (ctypes.c_char_p * 24)()
        n = ctypes.c_int()
        acc = {}
        for _ in range(reps):
            _lib.check(L.dftg_fock_build_profile(g.handle, vp(dP), ms, names, 24, ctypes.byref(n)))
            for i in range(n.value):
                acc.setdefault(names[i].decode(), []).append(ms[i])
        phases = {k: float(np.mean(v)) for k, v in acc.items()}
    npad = (npts + 127) // 128 * 128
    # operand bytes the mixed step streams: density (four BF16 slices of phi and the
    # FP64 amplitudes of its epilogue), the c phi operand pass (FP32 phi in, three
    # BF16 slices out), the contraction (three BF16 slices each of phi and c phi),
    # and the point arrays (rho, w, c)
    alg = (8 + 8 + 4 + 6 + 12) * npad * nbf + 8 * npad * 3
    # tensor-core contraction (nbf > 128): 128 x 128 tiles of the upper block triangle,
    # six BF16 slice products per tile and 16-point K step; operands three BF16 slices
    # of phi and of c phi, each streamed from HBM (L2 shares them between tiles)
    nrb = (nbf + 127) // 128
    ntiles = nrb * (nrb + 1) // 2
    tt_flop = 6 * 2 * npad * 128 * 128 * ntiles
    tt_bytes = 2 * 3 * 2 * npad * nrb * 128
    # tensor-core density (nbf > 80): 128-point tiles x 128-column blocks of Phi P, K = all
    # functions in 32-function stages, ten BF16 slice products per 16-function step
    nks = (nbf + 31) // 32
    dt_flop = 10 * 2 * npad * 128 * nrb * 32 * nks
    density_tc = None
    if "density" in phases and phases["density"] > 0:
        t = phases["density"] * 1e-3
        _, bf16, src = _peaks()
        density_tc = {"kernel": "k_density_tt (with the per-build P slicing)", "ms": phases["density"],
                      "bf16_tflops": dt_flop / t / 1e12, "bf16_peak_tflops": bf16,
                      "tensor_frac": (dt_flop / t / 1e12) / bf16 if bf16 else None, "peak_source": src}
    contract_tc = None
    if "contract" in phases and phases["contract"] > 0:
        t = phases["contract"] * 1e-3
        _, bf16, src = _peaks()
        contract_tc = {"kernel": "k_contract_tt", "tiles": ntiles, "ms": phases["contract"],
                       "bf16_tflops": tt_flop / t / 1e12, "bf16_peak_tflops": bf16,
                       "tensor_frac": (tt_flop / t / 1e12) / bf16 if bf16 else None,
                       "operand_GBps": tt_bytes / t / 1e9, "peak_source": src,
                       "operand_kernel_ms": phases.get("contract_operand")}
    out = {"workload": "synthetic: %d points, %d s/p/d primitives, P = C C^T (C %d x %d)" % (npts, nbf, nbf, nocc),
           "fp64_ms_per_step": ms64, "mixed_ms_per_step": msmx, "speedup": ms64 / msmx,
           "E_xc_fp64": float(s64[0]), "dE_xc_rel": abs(float(sm[0] - s64[0])) / abs(float(s64[0])),
           "max_dXC_rel": float(np.abs(xcm - xc64).max() / np.abs(xc64).max()),
           "max_drho_rel": float(np.abs(rhom - rho64).max() / np.abs(rho64).max()),
           "mixed_path": "tcgen05 tensor cores: density Phi P over 128-point x 128-column tiles (four BF16 slices of phi and of P, ten slice products) and XC contraction over 128 x 128 tiles (three BF16 slices of phi and of c phi, six slice products); exact integer leading products, double-float epilogues",
           "phases_ms_mixed": phases, "density_tensor_core": density_tc, "contract_tensor_core": contract_tc,
           "mixed_alg_bytes": alg, "mixed_GBps_over_alg_bytes": alg / (msmx * 1e-3) / 1e9, "setup_s": setup_s}
    g.close()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint (forces) workload")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-geometries workload")
    ap.add_argument("--no-synthetic", action="store_true", help="skip the synthetic contraction workload")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    world = _env_int("WORLD_SIZE", 1)
    rank = _env_int("RANK", 0)
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.init_process_group("nccl")
    if args.impl == "reference":
        out = run_reference(args, rank)
    else:
        out = run_ours(args, rank, world)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if world > 1 and args.impl == "ours":
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()

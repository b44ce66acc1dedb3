"""Batched builds on a caller's stream: ordering and timing.

A batch launched with dftg_batch_fock_build_device(..., stream) forks its
per-context branches from `stream` and joins them back into it, so work the
caller queues on that stream before the call (zeroing the outputs) precedes the
batch, and CUDA events recorded on it around the call bracket the whole batch.

Checks: outputs zeroed on the stream without any host synchronisation are
overwritten by the batch; the event time of a run of replays is at least 0.8 of
the host wall-clock time of the same replays synchronised on both sides, less
0.3 ms of launch and synchronisation overhead (events that missed the work
would read a few microseconds)."""
import time

import numpy as np
import pytest

from dftcxx_gb300.molecule import Molecule, small_molecule

pytestmark = pytest.mark.gpu


def test_batch_on_caller_stream_is_ordered_and_timed(gpu_lib):
    import torch
    from dftcxx_gb300.grid import MolecularGrid, Batch
    names = ["C6H6", "C2H6", "H2O", "NH3", "CH4", "CO", "C6H6", "N2"]
    grids, Pd, outs = [], [], []
    dev = torch.device("cuda")
    rng = np.random.default_rng(3)
    for i, name in enumerate(names):
        Z, xyz = small_molecule(name)
        mol = Molecule(Z, xyz, "p631" if i % 2 == 0 else "sto3g")
        grids.append(MolecularGrid(mol, 50, 10, 8, precision="mixed"))
        C = rng.normal(0, 0.2, size=(mol.nbf, mol.nelec // 2))
        Pd.append(torch.from_numpy(np.asfortranarray(C @ C.T).ravel(order="F").copy()).to(dev))
        outs.append(torch.zeros(2 * mol.nbf * mol.nbf, dtype=torch.float64, device=dev))
    b = Batch(grids)
    stream = torch.cuda.Stream()
    Js = [o[:g.nbf * g.nbf] for g, o in zip(grids, outs)]
    XCs = [o[g.nbf * g.nbf:] for g, o in zip(grids, outs)]
    torch.cuda.synchronize()
    run = lambda: b.build(Pd, Js, XCs, None, stream=stream.cuda_stream)
    run(); run()                                  # eager, then captured
    with torch.cuda.stream(stream):
        for o in outs:
            o.zero_()                             # queued on the caller's stream, no host wait
    run()
    stream.synchronize()
    assert all(bool(o.abs().max() > 0) for o in outs)

    reps = 5
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        run()
    e1.record(stream)
    e1.synchronize()
    t_ev = e0.elapsed_time(e1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        run()
    stream.synchronize()
    t_wall = (time.perf_counter() - t0) * 1e3
    assert t_ev >= 0.8 * t_wall - 0.3, (t_ev, t_wall)
    b.close()
    for g in grids:
        g.close()


def test_default_streams_are_rejected(gpu_lib):
    """The builds are captured into CUDA graphs, which the legacy and
    per-thread default streams do not allow: dftg_set_stream and the batch
    call reject them with DFTG_ERR_ARG instead of failing inside a capture."""
    import ctypes
    import torch
    from dftcxx_gb300 import _lib
    from dftcxx_gb300.grid import MolecularGrid, Batch
    Z, xyz = small_molecule("H2O")
    g = MolecularGrid(Molecule(Z, xyz, "sto3g"), 16, 4, 6, precision="fp64")
    L = _lib.load()
    for s in (1, 2):                       # cudaStreamLegacy, cudaStreamPerThread
        assert L.dftg_set_stream(g.handle, ctypes.c_void_p(s)) == _lib.DFTG_ERR_ARG
        assert b"default streams" in L.dftg_last_error()
    b = Batch([g])
    P = torch.zeros(g.nbf * g.nbf, dtype=torch.float64, device="cuda")
    arr = (ctypes.c_void_p * 1)(P.data_ptr())
    assert L.dftg_batch_fock_build_device(b._h, arr, None, None, None, ctypes.c_void_p(1)) == _lib.DFTG_ERR_ARG
    b.close()
    g.close()

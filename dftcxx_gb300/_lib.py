"""ctypes binding of ``libdftg.so`` (include/dftg.h).

The library is the product: every computation of the grid Fock build runs in
its CUDA kernels.  Loading fails loudly when the library has not been built;
there is no CPU fallback.
"""
import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libdftg.so")

DFTG_OK = 0
DFTG_ERR_ARG = 1
DFTG_ERR_CUDA = 2
DFTG_ERR_NONFINITE = 3
DFTG_ERR_STATE = 4
DFTG_ERR_NOMEM = 5
DFTG_ERR_TIMEOUT = 6
DFTG_PREC_FP64 = 0
DFTG_PREC_MIXED = 1
DFTG_LEBEDEV_302 = 11
NOALLOC_SCRATCH_BYTES = 16 * 1024 * 1024
NOALLOC_MAX_NBF = 1024

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)


class Molecule(ctypes.Structure):
    _fields_ = [("natoms", ctypes.c_int), ("Z", _ip), ("xyz", _dp)]


class Basis(ctypes.Structure):
    _fields_ = [("nbf", ctypes.c_int), ("bf_atom", _ip), ("bf_lmn", _ip), ("bf_nprim", _ip),
                ("prim_alpha", _dp), ("prim_coef", _dp)]


class GridParams(ctypes.Structure):
    _fields_ = [("radial_points", ctypes.c_int), ("lebedev_order", ctypes.c_int), ("lmax", ctypes.c_int),
                ("device", ctypes.c_int)]


class Points(ctypes.Structure):
    _fields_ = [("npts", ctypes.c_size_t), ("xyz", _dp), ("w", _dp)]


class ScfParams(ctypes.Structure):
    _fields_ = [("nelec", ctypes.c_int), ("alpha", ctypes.c_double), ("tol", ctypes.c_double),
                ("min_iter", ctypes.c_int), ("max_iter", ctypes.c_int), ("refine_steps", ctypes.c_int)]


SCF_MAX_NBF = 160
SCF_MAX_ITER = 1000
SCF_P, SCF_J, SCF_XC, SCF_H, SCF_X, SCF_EPS, SCF_COCC, SCF_HISTORY, SCF_DIAG, SCF_STATE = range(10)
SCF_HIST_W = 6


class DftgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("dftg error %d: %s" % (code, msg))
        self.code = code


# (name, argtypes); every entry point returns int except dftg_last_error
SIGNATURES = {
    "dftg_create": [ctypes.POINTER(Molecule), ctypes.POINTER(Basis), ctypes.POINTER(GridParams),
                    ctypes.POINTER(ctypes.c_void_p)],
    "dftg_create_cells": [ctypes.POINTER(Molecule), ctypes.POINTER(Basis), ctypes.POINTER(GridParams), ctypes.c_int,
                          ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)],
    "dftg_shard_blob_size": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t), _ip, _ip],
    "dftg_shard_density": [ctypes.c_void_p, _dp, _dp],
    "dftg_shard_multipoles": [ctypes.c_void_p, ctypes.c_double, _dp, ctypes.c_size_t],
    "dftg_shard_finish": [ctypes.c_void_p, _dp, ctypes.c_size_t, _dp, _dp, _dp],
    "dftg_destroy": [ctypes.c_void_p],
    "dftg_grid_size": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t)],
    "dftg_nbf": [ctypes.c_void_p, _ip],
    "dftg_set_precision": [ctypes.c_void_p, ctypes.c_int],
    "dftg_set_stream": [ctypes.c_void_p, ctypes.c_void_p],
    "dftg_set_precision_mask": [ctypes.c_void_p, ctypes.c_uint],
    "dftg_set_density": [ctypes.c_void_p, _dp],
    "dftg_correct_densities": [ctypes.c_void_p, _dp],
    "dftg_calculate_density": [ctypes.c_void_p, _dp],
    "dftg_calculate_hartree_potential": [ctypes.c_void_p, _dp],
    "dftg_calculate_xc": [ctypes.c_void_p, _dp, _dp],
    "dftg_fock_build": [ctypes.c_void_p, _dp, _dp, _dp, _dp, _dp],
    "dftg_fock_build_device": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
    "dftg_fock_build_profile": [ctypes.c_void_p, ctypes.c_void_p, _dp, ctypes.POINTER(ctypes.c_char_p), ctypes.c_int,
                                ctypes.POINTER(ctypes.c_int)],
    "dftg_get_weights": [ctypes.c_void_p, _dp, ctypes.c_size_t],
    "dftg_get_becke_weights": [ctypes.c_void_p, _dp, ctypes.c_size_t],
    "dftg_get_densities": [ctypes.c_void_p, _dp, ctypes.c_size_t],
    "dftg_get_amplitudes": [ctypes.c_void_p, _dp, ctypes.c_size_t],
    "dftg_get_positions": [ctypes.c_void_p, _dp, ctypes.c_size_t],
    "dftg_get_potential": [ctypes.c_void_p, _dp, ctypes.c_size_t],
    "dftg_one_electron": [ctypes.c_void_p, _dp, _dp, _dp],
    "dftg_contract_noalloc": [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p,
                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
    "dftg_nuclear_repulsion": [ctypes.c_void_p, _dp],
    "dftg_get_energies": [ctypes.c_void_p, _dp, _dp, _dp],
    "dftg_backward": [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, _dp, _dp],
    "dftg_backward_profile": [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, _dp, ctypes.POINTER(ctypes.c_char_p),
                              ctypes.c_int, ctypes.POINTER(ctypes.c_int)],
    "dftg_backward_device": [ctypes.c_void_p, ctypes.c_double, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p],
    "dftg_create_points": [ctypes.POINTER(Points), ctypes.POINTER(Molecule), ctypes.POINTER(Basis), ctypes.c_int,
                           ctypes.POINTER(ctypes.c_void_p)],
    "dftg_xc_build": [ctypes.c_void_p, _dp, _dp, _dp, _dp],
    "dftg_xc_build_device": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
    "dftg_get_launch_shape": [ctypes.c_void_p, _ip, ctypes.c_int],
    "dftg_set_launch_shape": [ctypes.c_void_p, _ip, ctypes.c_int],
    "dftg_autotune": [ctypes.c_void_p, ctypes.c_int, _dp],
    "dftg_batch_autotune": [ctypes.c_void_p, ctypes.c_int, _dp],
    "dftg_batch_create": [ctypes.POINTER(ctypes.c_void_p), ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)],
    "dftg_batch_destroy": [ctypes.c_void_p],
    "dftg_batch_set_mode": [ctypes.c_void_p, ctypes.c_int],
    "dftg_batch_get_mode": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)],
    "dftg_batch_status": [ctypes.c_void_p],
    "dftg_batch_selftest_wait": [ctypes.c_void_p, ctypes.c_double],
    "dftg_batch_fock_build_device": [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                                     ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(ctypes.c_void_p),
                                     ctypes.c_void_p],
    "dftg_eri_coulomb": [ctypes.c_void_p, _dp, _dp],
    "dftg_selftest_wait": [ctypes.c_void_p, ctypes.c_double],
    "dftg_eri_list": [ctypes.c_void_p, _dp, ctypes.c_size_t],
    "dftg_scf_init": [ctypes.c_void_p, ctypes.POINTER(ScfParams)],
    "dftg_scf_run": [ctypes.c_void_p, _dp, _ip],
    "dftg_scf_step": [ctypes.c_void_p, _dp, _ip],
    "dftg_scf_get": [ctypes.c_void_p, ctypes.c_int, _dp, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t)],
}

_lib = None


def load(path=LIB_PATH):
    """Load the CUDA library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise RuntimeError("libdftg.so not built (run dftcxx_gb300.build.build()); "
                           "the grid Fock build has no CPU fallback")
    L = ctypes.CDLL(path)
    for name, args in SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = ctypes.c_int
    L.dftg_last_error.restype = ctypes.c_char_p
    L.dftg_last_error.argtypes = []
    _lib = L
    return L


def check(rc):
    if rc != DFTG_OK:
        raise DftgError(rc, load().dftg_last_error().decode(errors="replace"))

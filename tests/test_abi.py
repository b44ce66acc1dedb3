"""The C ABI (include/dftg.h) without a GPU: the library loads, exports every
declared entry point, and rejects bad arguments before touching the device."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "dftg.h")


def _declared():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+char\s*\*|int)\s*(dftg_\w+)\s*\(", text, flags=re.M)))


def _defines():
    out = {}
    for name, val in re.findall(r"^#define\s+(DFTG_\w+)\s+(\d+)u?\b", open(HEADER).read(), flags=re.M):
        out[name] = int(val)
    return out


@pytest.fixture(scope="module")
def lib():
    from dftcxx_gb300 import build, _lib
    build.build()
    return _lib.load()


def test_header_declares_the_entry_points():
    names = _declared()
    for n in ("dftg_create", "dftg_destroy", "dftg_set_density", "dftg_correct_densities",
              "dftg_calculate_hartree_potential", "dftg_calculate_xc", "dftg_fock_build",
              "dftg_get_amplitudes", "dftg_one_electron", "dftg_contract_noalloc"):
        assert n in names
    assert len(names) >= 25


def test_library_exports_every_declared_symbol(lib):
    from dftcxx_gb300 import _lib
    for name in _declared():
        assert hasattr(lib, name), name
        if name != "dftg_last_error":
            assert name in _lib.SIGNATURES, name


def test_python_constants_match_header():
    from dftcxx_gb300 import _lib, grid
    d = _defines()
    assert _lib.NOALLOC_SCRATCH_BYTES == 16 * 1024 * 1024 and _lib.NOALLOC_MAX_NBF == d["DFTG_NOALLOC_MAX_NBF"]
    for k in ("DFTG_OK", "DFTG_ERR_ARG", "DFTG_ERR_CUDA", "DFTG_ERR_NONFINITE", "DFTG_ERR_STATE",
              "DFTG_ERR_NOMEM", "DFTG_ERR_TIMEOUT", "DFTG_PREC_FP64", "DFTG_PREC_MIXED", "DFTG_LEBEDEV_302"):
        assert getattr(_lib, k) == d[k], k
    assert grid.MolecularGrid.MIX_BITS == {
        "density": d["DFTG_MIX_DENSITY"], "lda": d["DFTG_MIX_LDA"], "multipole": d["DFTG_MIX_MULTIPOLE"],
        "cross": d["DFTG_MIX_CROSS"], "contract": d["DFTG_MIX_CONTRACT"]}


def _structs(Z, xyz, nbf=1, lmn=(0, 0, 0), alpha=1.0, nrad=16, leb=5, lmax=4, bf_atom=0):
    from dftcxx_gb300 import _lib
    keep = {}
    keep["Z"] = np.asarray(Z, dtype=np.int32)
    keep["xyz"] = np.ascontiguousarray(xyz, dtype=np.float64)
    keep["bf_atom"] = np.full(nbf, bf_atom, dtype=np.int32)
    keep["bf_lmn"] = np.tile(np.asarray(lmn, dtype=np.int32), nbf)
    keep["bf_nprim"] = np.ones(nbf, dtype=np.int32)
    keep["alpha"] = np.full(nbf, alpha)
    keep["coef"] = np.ones(nbf)
    ip = ctypes.POINTER(ctypes.c_int)
    dp = ctypes.POINTER(ctypes.c_double)
    m = _lib.Molecule(len(Z), keep["Z"].ctypes.data_as(ip), keep["xyz"].ctypes.data_as(dp))
    b = _lib.Basis(nbf, keep["bf_atom"].ctypes.data_as(ip), keep["bf_lmn"].ctypes.data_as(ip),
                   keep["bf_nprim"].ctypes.data_as(ip), keep["alpha"].ctypes.data_as(dp),
                   keep["coef"].ctypes.data_as(dp))
    g = _lib.GridParams(nrad, leb, lmax, 0)
    return m, b, g, keep


def _create(lib, m, b, g):
    h = ctypes.c_void_p()
    rc = lib.dftg_create(ctypes.byref(m), ctypes.byref(b), ctypes.byref(g), ctypes.byref(h))
    return rc, h, lib.dftg_last_error().decode()


@pytest.mark.parametrize("case,code,msg", [
    ("natoms0", "DFTG_ERR_ARG", "natoms"),
    ("Z0", "DFTG_ERR_ARG", "Z[0]"),
    ("Z19", "DFTG_ERR_ARG", "Z[0]"),
    ("nan", "DFTG_ERR_NONFINITE", "not finite"),
    ("coincide", "DFTG_ERR_ARG", "coincide"),
    ("nrad", "DFTG_ERR_ARG", "radial_points"),
    ("leb", "DFTG_ERR_ARG", "lebedev_order"),
    ("lmax", "DFTG_ERR_ARG", "lmax"),
    ("bf_atom", "DFTG_ERR_ARG", "bf_atom"),
    ("ang", "DFTG_ERR_ARG", "angular momentum"),
    ("alpha", "DFTG_ERR_ARG", "exponent"),
])
def test_create_rejects_bad_input(lib, case, code, msg):
    from dftcxx_gb300 import _lib
    Z, xyz = [1, 1], [[0.0, 0.0, 0.0], [0.0, 0.0, 1.4]]
    kw = {}
    if case == "natoms0":
        Z, xyz = [], np.zeros((0, 3))
    elif case == "Z0":
        Z = [0, 1]
    elif case == "Z19":
        Z = [19, 1]
    elif case == "nan":
        xyz = [[0.0, 0.0, float("nan")], [0.0, 0.0, 1.4]]
    elif case == "coincide":
        xyz = [[0.0, 0.0, 0.0], [0.0, 0.0, 0.0]]
    elif case == "nrad":
        kw["nrad"] = 4
    elif case == "leb":
        kw["leb"] = 12
    elif case == "lmax":
        kw["lmax"] = 17
    elif case == "bf_atom":
        kw["bf_atom"] = 2
    elif case == "ang":
        kw["lmn"] = (3, 2, 0)
    elif case == "alpha":
        kw["alpha"] = -1.0
    m, b, g, keep = _structs(Z, xyz, **kw)
    rc, h, err = _create(lib, m, b, g)
    assert rc == getattr(_lib, code), (rc, err)
    assert msg in err
    assert not h.value


def test_create_null_arguments(lib):
    from dftcxx_gb300 import _lib
    h = ctypes.c_void_p()
    assert lib.dftg_create(None, None, None, ctypes.byref(h)) == _lib.DFTG_ERR_ARG
    assert lib.dftg_create(None, None, None, None) == _lib.DFTG_ERR_ARG


def test_null_context_is_rejected_everywhere(lib):
    from dftcxx_gb300 import _lib
    d = ctypes.c_double()
    n = ctypes.c_size_t()
    i = ctypes.c_int()
    buf = (ctypes.c_double * 4)()
    calls = [
        lambda: lib.dftg_grid_size(None, ctypes.byref(n)),
        lambda: lib.dftg_nbf(None, ctypes.byref(i)),
        lambda: lib.dftg_set_precision(None, 0),
        lambda: lib.dftg_set_precision_mask(None, 0),
        lambda: lib.dftg_set_stream(None, None),
        lambda: lib.dftg_set_density(None, buf),
        lambda: lib.dftg_correct_densities(None, ctypes.byref(d)),
        lambda: lib.dftg_calculate_density(None, ctypes.byref(d)),
        lambda: lib.dftg_calculate_hartree_potential(None, buf),
        lambda: lib.dftg_calculate_xc(None, buf, ctypes.byref(d)),
        lambda: lib.dftg_fock_build(None, buf, buf, buf, ctypes.byref(d), ctypes.byref(d)),
        lambda: lib.dftg_fock_build_device(None, None, None, None, None),
        lambda: lib.dftg_get_weights(None, buf, 4),
        lambda: lib.dftg_get_becke_weights(None, buf, 4),
        lambda: lib.dftg_get_densities(None, buf, 4),
        lambda: lib.dftg_get_amplitudes(None, buf, 4),
        lambda: lib.dftg_get_positions(None, buf, 4),
        lambda: lib.dftg_get_potential(None, buf, 4),
        lambda: lib.dftg_get_energies(None, ctypes.byref(d), ctypes.byref(d), ctypes.byref(d)),
        lambda: lib.dftg_one_electron(None, buf, buf, buf),
        lambda: lib.dftg_nuclear_repulsion(None, ctypes.byref(d)),
    ]
    for call in calls:
        assert call() == _lib.DFTG_ERR_ARG
    assert lib.dftg_destroy(None) == _lib.DFTG_OK


def test_contract_noalloc_rejects_before_device_use(lib):
    from dftcxx_gb300 import _lib
    dummy = ctypes.c_void_p(0x1000)      # never dereferenced: the size checks come first
    rc = lib.dftg_contract_noalloc(dummy, 64, 64, _lib.NOALLOC_MAX_NBF + 1, dummy, dummy, dummy, dummy, None)
    assert rc == _lib.DFTG_ERR_ARG
    assert "no-allocation limit" in lib.dftg_last_error().decode()
    assert lib.dftg_contract_noalloc(None, 64, 64, 8, dummy, dummy, dummy, dummy, None) == _lib.DFTG_ERR_ARG
    assert lib.dftg_contract_noalloc(dummy, 32, 64, 8, dummy, dummy, dummy, dummy, None) == _lib.DFTG_ERR_ARG
    assert lib.dftg_contract_noalloc(dummy, 64, 64, 8, dummy, dummy, None, None, None) == _lib.DFTG_ERR_ARG


def test_product_has_no_cpu_fallback(monkeypatch, tmp_path):
    """Loading fails loudly when the CUDA library is absent."""
    from dftcxx_gb300 import _lib
    monkeypatch.setattr(_lib, "_lib", None)
    with pytest.raises(RuntimeError, match="no CPU fallback"):
        _lib.load(str(tmp_path / "missing.so"))

"""The C-ABI library builds, loads without a GPU, exports every function
that include/lbm_gb300.h declares, and its ctypes struct mirror matches the
C layout (offsets checked with gcc)."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

from lbm_gb300 import _build, _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "lbm_gb300.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(lbm_[a-z0-9_]+)\s*\(", text)))


def test_library_builds_and_loads():
    path = _build.build()
    assert os.path.exists(path)
    L = ctypes.CDLL(path)
    assert L.lbm_abi_version() == 2


def test_every_declared_symbol_is_exported():
    _build.build()
    L = ctypes.CDLL(_build.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # and the Python binding knows all of them
    assert sorted(set(names) - set(_lib.exported_symbols())) == []


@pytest.mark.parametrize("cls,cname", [(_lib.Problem, "lbm_problem"),
                                        (_lib.BatchConfig, "lbm_batch_config"),
                                        (_lib.Adjoint, "lbm_adjoint")])
def test_struct_layout_matches_c(cls, cname):
    fields = [f[0] for f in cls._fields_]
    src = ['#include <stdio.h>', '#include <stddef.h>', '#include "lbm_gb300.h"', "int main(void){"]
    src.append('printf("size %%zu\\n", sizeof(%s));' % cname)
    for f in fields:
        src.append('printf("%s %%zu\\n", offsetof(%s, %s));' % (f, cname, f))
    src.append("return 0;}")
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "t.c")
        open(c, "w").write("\n".join(src))
        exe = os.path.join(d, "t")
        subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe])
        out = subprocess.check_output([exe]).decode().split("\n")
    got = dict(line.split() for line in out if line.strip())
    assert int(got["size"]) == ctypes.sizeof(cls)
    for f in fields:
        assert int(got[f]) == getattr(cls, f).offset, f


def test_scratch_bytes_is_host_only():
    L = _lib.load()
    P = _lib.Problem()
    P.nx, P.ny, P.n_special, P.n_links = 10, 10, 36, 5
    n = L.lbm_problem_scratch_bytes(ctypes.byref(P))
    assert n >= 8 * (24 * 36 + 2 * 5)


def test_argument_errors_are_reported_without_gpu_work():
    """Invalid arguments fail in the host checks, before any CUDA call."""
    L = _lib.load()
    assert L.lbm_macro_f64(None, None, None, 2, 2, None) == _lib.LBM_ERR_ARG
    assert b"lattice" in L.lbm_last_error_string()
    P = _lib.Problem()
    assert L.lbm_advance(ctypes.byref(P), 1, 0, 1, 0, 0, None) == _lib.LBM_ERR_ARG
    with pytest.raises(_lib.LbmError):
        _lib.call("lbm_zou_he_f64", 9, None, None, None, None, None, 8, 8, None)


def test_batch_config_checked_without_gpu_work():
    """A batch configuration outside its documented ranges (tile_rounds
    1..64, vec_bytes 8 or 16, persistent 0 or 1) is refused by the host
    checks of lbm_batch_create."""
    L = _lib.load()
    P = _lib.Problem()
    good = dict(bulk_threads=128, bulk_blocks_per_sm=8, special_blocks_per_sm=8,
                scalar_tile_cells=2048, persistent=0, vec_bytes=8, tile_rounds=4)
    for key, bad in (("tile_rounds", 0), ("tile_rounds", 65), ("vec_bytes", 4),
                     ("persistent", 2), ("bulk_threads", 48)):
        cfg = _lib.BatchConfig(**dict(good, **{key: bad}))
        h = ctypes.c_void_p()
        rc = L.lbm_batch_create(ctypes.byref(h), ctypes.byref(P), 1, ctypes.byref(cfg))
        assert rc == _lib.LBM_ERR_ARG, (key, bad)
        assert b"bad config" in L.lbm_last_error_string()
        assert not h.value

"""The C ABI library loads, exports every symbol include/*.h declares, and
rejects bad calls without a device (CPU only; no compute call is made)."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import pytest

import grudon_gb300 as g
from grudon_gb300 import _ffi

ROOT = Path(__file__).resolve().parent.parent


def declared_symbols():
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names.update(re.findall(r"\b(grd_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_every_declared_symbol_is_exported():
    out = subprocess.run(["nm", "-D", "--defined-only", str(_ffi.LIB_PATH)], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (grd_\w+)", out))
    missing = [s for s in declared_symbols() if s not in exported]
    assert not missing, missing
    # and every declared symbol has a ctypes signature
    assert set(declared_symbols()) <= set(_ffi.SIGNATURES), set(declared_symbols()) - set(_ffi.SIGNATURES)


def test_version_and_device_count():
    assert b"sm_103a" in g.lib().grd_version()
    assert g.device_count() >= 0


def test_ctx_create_argument_errors():
    lib = g.lib()
    G = g.Graph.rmat(6, 4)
    ctx = C.c_void_p()
    csr = G.csr_struct()
    assert lib.grd_ctx_create(None, None, 1, 1, 0, C.byref(ctx)) == _ffi.GRD_E_INVALID
    assert lib.grd_ctx_create(C.byref(csr), None, 2, 1, 0, C.byref(ctx)) == _ffi.GRD_E_INVALID
    assert b"num_compute" in lib.grd_create_error()
    assert lib.grd_ctx_create(C.byref(csr), None, 1, 1, 0, None) == _ffi.GRD_E_INVALID


@pytest.mark.skipif(g.device_count() > 0, reason="checks the no-device path")
def test_no_device_fails_loudly():
    G = g.Graph.rmat(6, 4)
    with pytest.raises(g.GrdError) as e:
        g.Context(G)
    assert e.value.code == _ffi.GRD_E_CUDA
    assert "no CUDA device" in str(e.value)


def test_null_ctx_calls_are_rejected():
    lib = g.lib()
    assert lib.grd_init(None) == _ffi.GRD_E_INVALID
    assert lib.grd_run(None, 0, None) == _ffi.GRD_E_INVALID
    assert lib.grd_update(None, None) == _ffi.GRD_E_INVALID
    assert lib.grd_set_algo(None, 0, None) == _ffi.GRD_E_INVALID
    lib.grd_ctx_destroy(None)


def test_cli_builds_and_validates_flags():
    cli = ROOT / "grudon_gb300" / "_build" / "grudon"
    assert cli.exists()
    r = subprocess.run([str(cli)], capture_output=True, text=True)
    assert r.returncode == 1 and "graph path" in r.stderr
    r = subprocess.run([str(cli), "-g", "x.gr", "-c", "1"], capture_output=True, text=True)
    assert r.returncode == 1 and "mirror nodes" in r.stderr

"""CPU tests of the C ABI: the library builds for sm_103a, loads, exports every
symbol include/seidart_gb300.h declares, and rejects bad configurations on the
host (no device work is done here)."""
import ctypes as C
import re
from pathlib import Path

import pytest

from seidart_gb300 import _lib, build
from seidart_gb300._lib import SfdConfig

HEADER = Path(__file__).resolve().parents[1] / "include" / "seidart_gb300.h"


@pytest.fixture(scope="module")
def L():
    build.build()
    return _lib.lib()


def test_exports_every_declared_symbol(L):
    declared = set(re.findall(r"\b(sfd_\w+)\s*\(", HEADER.read_text()))
    assert declared, "no declarations parsed"
    assert declared == set(_lib.EXPORTS)
    for name in declared:
        assert hasattr(L, name), name


def test_counts(L):
    assert L.sfd_model_planes(_lib.SEISMIC2) == 9
    assert L.sfd_model_planes(_lib.SEISMIC25) == 25
    assert L.sfd_model_planes(_lib.ELECTROMAG2) == 6
    assert L.sfd_model_planes(_lib.ELECTROMAG25) == 12
    assert L.sfd_num_fields(_lib.SEISMIC25) == 9 and L.sfd_num_channels(_lib.SEISMIC25) == 3
    assert L.sfd_num_memory(_lib.SEISMIC2) == 12 and L.sfd_num_memory(_lib.ELECTROMAG25) == 12
    assert L.sfd_version() >= 100


def _cfg(**kw):
    base = dict(kind=_lib.ELECTROMAG2, nx=64, ny=1, nz=48, npml=8, nstep=100, nrec=4, flags=0,
                dx=0.05, dy=0.05, dz=0.05, dt=1e-10)
    base.update(kw)
    return SfdConfig(**base)


def test_state_bytes(L):
    n = C.c_size_t()
    assert L.sfd_state_bytes(C.byref(_cfg()), C.byref(n)) == 0
    assert n.value > 3 * 64 * 48 * 4
    n3 = C.c_size_t()
    assert L.sfd_state_bytes(C.byref(_cfg(kind=_lib.SEISMIC25, ny=30)), C.byref(n3)) == 0
    assert n3.value > 9 * 64 * 30 * 48 * 4


@pytest.mark.parametrize("bad,frag", [
    (dict(kind=9), "kind"),
    (dict(ny=5), "ny = 1"),
    (dict(nx=10), "too small"),
    (dict(npml=0), "npml"),
    (dict(dt=0.0), "positive"),
    (dict(flags=4), "flags"),
    (dict(kind=_lib.SEISMIC25, ny=4), "ny="),
])
def test_bad_config_rejected(L, bad, frag):
    n = C.c_size_t()
    rc = L.sfd_state_bytes(C.byref(_cfg(**bad)), C.byref(n))
    assert rc == _lib.SFD_ERR_BAD_ARG
    assert frag in L.sfd_last_error().decode()


def test_create_rejects_null_buffer(L):
    h = C.c_void_p()
    rc = L.sfd_create(C.byref(_cfg()), None, 0, None, C.byref(h))
    assert rc == _lib.SFD_ERR_BAD_ARG and not h.value


def test_library_sources_never_allocate_device_memory():
    """The library allocates no device memory (callers pass every buffer; the
    allocation-free entry point relies on it): no CUDA allocation or free call
    appears in its sources outside comments."""
    import re
    csrc = Path(__file__).resolve().parent.parent / "seidart_gb300" / "csrc"
    pat = re.compile(r"\b(cudaMalloc\w*|cudaFree\w*|cuMemAlloc\w*|cuMemFree\w*)\s*\(")
    for f in sorted(csrc.glob("*.c*")) + sorted(csrc.glob("*.h")):
        code = re.sub(r"//[^\n]*|/\*.*?\*/", "", f.read_text(), flags=re.S)
        hits = pat.findall(code)
        assert not hits, f"{f.name} calls {hits}"

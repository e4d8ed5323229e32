"""CPU-side checks of the C ABI: the library loads without a GPU, exports exactly the
symbols include/bz.h declares, the ctypes layout of bz_params matches the header, and
argument validation rejects bad calls before anything is launched."""
import ctypes
import os
import re
import subprocess

import pytest

from boltzmann_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(ROOT, "include", "bz.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    names = re.findall(r"^[a-z_ ]*?[\w\*]+\s+\**(bz_\w+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(_lib.LIB_PATH):
        from boltzmann_gb300 import build
        build.build()
    return _lib.load()


def test_header_and_bindings_agree():
    assert header_functions() == _lib.exported_symbols()


def test_library_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (bz_\w+)", out))
    for name in header_functions():
        assert name in exported, name
        assert getattr(lib, name) is not None


def test_version(lib):
    assert b"sm_103a" in lib.bz_version()


def test_params_layout_matches_header(lib):
    # offsets of the C struct on LP64: 4 int32, 2 double, 5 double, 4 int32, 2 double, ptr, 2 u64, ptr
    P = _lib.BzParams
    assert P.L.offset == 16 and P.dt.offset == 32 and P.xs_mode.offset == 72
    assert P.xs_emin.offset == 88 and P.xs_table.offset == 104 and P.seed.offset == 112
    assert P.step_ptr.offset == 128 and ctypes.sizeof(P) == 136


def test_argument_validation_without_gpu(lib):
    p = _lib.BzParams()
    empty = _lib.Particles()
    # null pointers are rejected before any CUDA call
    rc = lib.bz_push_collide_f32(ctypes.byref(p), empty, None, 10, empty, 10, None, None, None, None, None, None, 0,
                                 None, None)
    assert rc == _lib.BZ_ERR_ARG
    rc = lib.bz_bin_f32(ctypes.byref(p), empty, None, 10, 1, None, 0.1, None, None, None, None, None, 0, None, None)
    assert rc == _lib.BZ_ERR_ARG
    assert lib.bz_poisson(2, 0.1, 1.0, 1.0, 1.0, 0.0, None, None, None, None, None, None, None, None) == \
        _lib.BZ_ERR_ARG
    assert lib.bz_push_workspace(1 << 20) >= 8 * 1024
    assert lib.bz_bin_workspace(1 << 20, 5000) > 6 * (1 << 20)


def test_missing_library_fails_loudly(monkeypatch, tmp_path):
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "libbz.so"))
    with pytest.raises(_lib.BzLibraryError):
        _lib.load()


def test_new_entry_points_validate_without_gpu(lib):
    """The placement, the checked binning and the in-place resampling reject bad calls
    before anything is launched; the workspace queries need no GPU."""
    p = _lib.BzParams()
    seg0 = _lib.Segments()
    empty = _lib.Particles()
    # null pointers
    assert lib.bz_seg_place_f32(seg0, empty, None, 0, seg0, None, 0, None, None, None) == _lib.BZ_ERR_ARG
    assert lib.bz_seg_bin_check_f32(ctypes.byref(p), seg0, 3, None, 0.1, None, None, None, None, None, 0.5, 3.0,
                                    None, None, 0, None, None) == _lib.BZ_ERR_ARG
    # in-place resampling with a scratch set of another geometry: refused on the host
    fake = ctypes.c_void_p(256)  # never dereferenced: the call returns before any launch
    cnt = ctypes.c_void_p(512)

    def seg(nseg, half):
        s = _lib.Segments()
        s.x = s.vx = s.vy = s.vz = s.w = fake
        s.counts = cnt
        s.nseg, s.half = nseg, half
        return s

    app = _lib.Particles(fake, fake, fake, fake, fake)
    q = _lib.BzParams()
    q.n_nodes = 17
    q.flags = _lib.RESAMPLE_IN_PLACE
    rc = lib.bz_seg_resample_f32(ctypes.byref(q), seg(4, 64), app, 100, seg(8, 64), 3, fake, fake, 0.1, 0.5, 3.0,
                                 0.6, fake, fake, fake, fake, None, None, None, fake, 1 << 30, None, fake, None)
    assert rc == _lib.BZ_ERR_ARG
    # the checked binning without targets: refused before anything runs
    q2 = _lib.BzParams()
    q2.n_nodes = 17
    rc = lib.bz_seg_bin_check_f32(ctypes.byref(q2), seg(4, 64), 3, fake, 0.1, fake, fake, fake, fake, None, 0.5, 3.0,
                                  None, fake, 1 << 30, fake, None)
    assert rc == _lib.BZ_ERR_ARG
    # workspace queries
    n = 1025
    assert lib.bz_seg_push_workspace_nodes(n) >= lib.bz_seg_push_workspace() + 8 * n
    assert lib.bz_push_workspace_fast_f32(1 << 20, n) >= 40 * (1 << 20)
    assert lib.bz_push_workspace_fast_f64(1 << 20, n) >= 80 * (1 << 20)
    assert lib.bz_seg_place_workspace(1000) >= lib.bz_seg_repack_workspace(1000)

"""Run the reference's own Python source (jfabell/boltzmann) on the CPU.

TEST INFRASTRUCTURE ONLY. This module is part of the oracle: it is imported by
the golden-vector generator under ``tests/golden`` and by nothing on the product
path. It needs the reference checkout on disk, so it only works where that
checkout exists (the build container); the vectors it produces are committed as
fixtures so that nothing at test time needs the reference itself.

How it works: the reference imports ``numba`` (``njit``, ``prange``, ``cuda.jit``,
``cuda.atomic.add``, ``cuda.to_device``) and ``cupy``. Neither is installed here,
so this module installs stand-ins in ``sys.modules`` before importing the
reference's modules, unmodified, from their own directory:

* ``numba.njit`` / ``prange``: identity decorator / ``range``; the CPU kernels
  (``kernels/EF_kernel_1D.py``, ``kernels/heavies_kernel_1D.py``) run as plain Python.
* ``numba.cuda.jit``: returns a launcher that runs the kernel body once per
  (block, thread) of the requested grid, serially, in block-major then
  thread order, with ``cuda.threadIdx/blockIdx/blockDim/gridDim`` set. Atomics are
  a read-then-add, so the order of atomic appends is the thread order, which makes
  the reference's nondeterministic appends (``electron_kernel_numba.py:218``,
  ``bin_particles.py:20``) deterministic: ascending particle index.
* ``cupy``: numpy-backed arrays of class ``CpArray``. Two CuPy behaviours the
  reference relies on are restated: (1) integer-array indexing wraps out-of-range
  indices (CuPy documents this difference from NumPy); (2) indexing that selects a
  single element returns a 0-d array, so a later use of it as an index is integer
  *array* indexing and wraps too. ``boltzmann.py:820-822`` depends on both.
* ``cupy.random``: a recorded generator. Every draw is appended to ``DRAWS`` so the
  golden generator can hand the exact same random numbers to the CUDA kernels.
  ``choice`` restates the inverse-CDF algorithm that CuPy 13.4.1
  (``RandomState.choice``, replace=True with ``p``) shares with NumPy's legacy
  generator: ``cdf = cumsum(p); cdf /= cdf[-1]; idx = searchsorted(cdf, u, 'right')``.
* the pybind11 module ``cuda_red`` (``kernels/reduction/cuda_reduction/kernels-new.cu``)
  is replaced by ``_cuda_red_calls``, a numpy restatement of ``reda`` + ``redcheck``
  (race-free: all coarse sums are formed before any is written back).
"""
from __future__ import annotations

import ctypes
import importlib
import math
import os
import sys
import types

import numpy as np

REFERENCE_ROOT = os.environ.get("BZ_REFERENCE_ROOT", "/root/reference")

# --------------------------------------------------------------------------------------
# cupy stand-in
# --------------------------------------------------------------------------------------


class _Ptr:
    def __init__(self, ptr):
        self.ptr = ptr


def _wrap_index(shape, idx):
    """CuPy wraps out-of-range integer-array indices; numpy raises. Restate CuPy."""
    if not isinstance(idx, tuple):
        idx = (idx,)
    out = []
    axis = 0
    for comp in idx:
        if isinstance(comp, np.ndarray) and comp.dtype.kind in "iu":
            out.append(np.asarray(comp) % shape[axis])
            axis += 1
        elif comp is None:
            out.append(comp)
        elif comp is Ellipsis:
            raise NotImplementedError("Ellipsis indexing is not used by the reference")
        else:
            out.append(comp)
            axis += 1
    return tuple(out)


class CpArray(np.ndarray):
    """numpy array with CuPy's indexing semantics and a ``.data.ptr`` attribute."""

    def __getitem__(self, idx):
        res = np.ndarray.__getitem__(self, _wrap_index(self.shape, idx))
        if not isinstance(res, np.ndarray):
            res = np.asarray(res).view(CpArray)
        return res

    def __setitem__(self, idx, val):
        np.ndarray.__setitem__(self, _wrap_index(self.shape, idx), val)

    @property
    def data(self):  # cupy.ndarray.data.ptr -> device pointer; here the host address
        return _Ptr(self.ctypes.data)

    def tofile(self, f):
        np.asarray(self).tofile(f)


class DevArray(np.ndarray):
    """What ``numba.cuda.to_device`` returns: an alias of the same memory whose
    element reads are plain Python scalars, as inside a Numba CUDA kernel."""

    def __getitem__(self, idx):
        res = np.ndarray.__getitem__(self, idx)
        if isinstance(res, np.ndarray):
            return res
        return res.item()


def _cp(a):
    if isinstance(a, CpArray):
        return a
    return np.asarray(a).view(CpArray)


class _Recorder:
    """Records every random draw: list of (name, ndarray)."""

    def __init__(self):
        self.draws = []
        self.gen = np.random.Generator(np.random.PCG64(12345))

    def reset(self, seed):
        self.gen = np.random.Generator(np.random.PCG64(seed))
        self.draws = []


DRAWS = _Recorder()


def _rand(*shape):
    u = DRAWS.gen.random(shape if shape else None)
    DRAWS.draws.append(("rand", np.array(u, dtype=np.float64)))
    return _cp(u)


def _mvn(mean, cov, size):
    cov = np.asarray(cov, dtype=np.float64)
    if not np.allclose(cov, np.diag(np.diag(cov))):
        raise NotImplementedError("only diagonal covariances appear in the reference")
    z = DRAWS.gen.standard_normal((size, len(mean)))
    x = np.asarray(mean, dtype=np.float64) + z * np.sqrt(np.diag(cov))
    DRAWS.draws.append(("multivariate_normal", x.copy()))
    return _cp(x)


def _choice(a, size=None, replace=True, p=None):
    if not replace or p is None:
        raise NotImplementedError("the reference only uses choice(replace=True, p=...)")
    a = np.asarray(a)
    p = np.asarray(p, dtype=np.float64)
    cdf = np.cumsum(p)
    cdf /= cdf[-1]
    u = DRAWS.gen.random(size)
    idx = np.searchsorted(cdf, u, side="right")
    DRAWS.draws.append(("choice_uniform", np.array(u, dtype=np.float64)))
    return _cp(a[idx])


def _seed(s):
    DRAWS.gen = np.random.Generator(np.random.PCG64(int(s) + 1_000_000))


def _shuffle(x):
    perm = DRAWS.gen.permutation(x.shape[0])
    np.ndarray.__setitem__(x, slice(None), np.asarray(x)[perm])


def _make_cupy():
    cp = types.ModuleType("cupy")
    cp.ndarray = CpArray
    cp.pi = math.pi
    cp.float64 = np.float64
    for name in ("zeros", "ones", "arange", "empty"):
        f = getattr(np, name)
        setattr(cp, name, (lambda f: lambda *a, **k: _cp(f(*a, **k)))(f))
    cp.array = lambda a, *x, **k: _cp(np.array(a, *x, **k))
    cp.asarray = lambda a, *x, **k: _cp(np.array(a, *x, **k))
    cp.asnumpy = lambda a: np.array(a)

    def _red(f):
        def g(a, *x, **k):
            return _cp(f(np.asarray(a), *x, **k))
        return g

    for name in ("sum", "cumsum", "max", "min", "sqrt", "multiply", "add", "divide", "abs"):
        setattr(cp, name, _red(getattr(np, name)))

    def where(cond, *args):
        if args:
            return _cp(np.where(np.asarray(cond), *[np.asarray(a) for a in args]))
        return tuple(_cp(r) for r in np.where(np.asarray(cond)))

    cp.where = where
    cp.searchsorted = lambda a, v, side="left": _cp(np.searchsorted(np.asarray(a), np.asarray(v), side=side))

    def unique(a, return_counts=False):
        if return_counts:
            u, c = np.unique(np.asarray(a), return_counts=True)
            return _cp(u), _cp(c)
        return _cp(np.unique(np.asarray(a)))

    cp.unique = unique

    rnd = types.ModuleType("cupy.random")
    rnd.rand = _rand
    rnd.multivariate_normal = _mvn
    rnd.choice = _choice
    rnd.seed = _seed
    rnd.shuffle = _shuffle
    cp.random = rnd

    cuda = types.ModuleType("cupy.cuda")

    class _Dev:
        def __init__(self, *a):
            pass

        def use(self):
            return self

    cuda.Device = _Dev
    runtime = types.ModuleType("cupy.cuda.runtime")
    runtime.setDevice = lambda *a: None
    cuda.runtime = runtime
    cp.cuda = cuda
    return cp, rnd, cuda, runtime


# --------------------------------------------------------------------------------------
# numba stand-in
# --------------------------------------------------------------------------------------


class _Dim:
    def __init__(self, x=0):
        self.x = x


def _make_numba():
    numba = types.ModuleType("numba")
    cuda = types.ModuleType("numba.cuda")

    def njit(*a, **k):
        if a and callable(a[0]) and not k:
            return a[0]
        return lambda f: f

    numba.njit = njit
    numba.jit = njit
    numba.prange = range

    class _Launcher:
        def __init__(self, fn):
            self.fn = fn

        def __getitem__(self, cfg):
            blocks, threads = int(cfg[0]), int(cfg[1])

            def launch(*args):
                cuda.blockDim = _Dim(threads)
                cuda.gridDim = _Dim(blocks)
                for b in range(blocks):
                    cuda.blockIdx = _Dim(b)
                    for t in range(threads):
                        cuda.threadIdx = _Dim(t)
                        self.fn(*args)

            return launch

    def jit(*a, **k):
        if a and callable(a[0]):
            return _Launcher(a[0])
        return lambda f: _Launcher(f)

    class _Atomic:
        @staticmethod
        def add(arr, idx, val):
            old = np.ndarray.__getitem__(arr, idx).item()
            np.ndarray.__setitem__(arr, idx, old + val)
            return old

    cuda.jit = jit
    cuda.atomic = _Atomic
    cuda.to_device = lambda a: np.asarray(a).view(DevArray) if not isinstance(a, DevArray) else a
    cuda.select_device = lambda *a: None
    cuda.threadIdx = _Dim()
    cuda.blockIdx = _Dim()
    cuda.blockDim = _Dim(1)
    cuda.gridDim = _Dim(1)
    numba.cuda = cuda
    return numba, cuda


# --------------------------------------------------------------------------------------
# cuda_red stand-in: restatement of kernels/reduction/cuda_reduction/kernels-new.cu
# --------------------------------------------------------------------------------------


def _cuda_red_calls(r, p, M, RM, dw, dv, dx, ptcl):
    """``calls`` (kernels-new.cu:76-132): ``reda`` then, when M/RM > 1, ``redcheck``.

    reda (kernels-new.cu:56-73): fine bin b = int(x[i] * float(M)); w[r*b+j] += v[r*i+j].
    The FP64 atomics are applied in ascending particle order.
    redcheck (kernels-new.cu:8-50): block k of ``bloks = ceil(M/RM)`` threads tree-sums
    fine bins k*bloks .. k*bloks+bloks-1 (``s = bloks/2, /2, ..`` halving, which drops
    elements when bloks is not a power of two) and writes the sum to w[r*k+j]. The
    reference does this in place across blocks (a race); here every block sum is formed
    from the unmodified fine bins first.
    """
    dw = np.asarray(dw).reshape(-1)
    dv = np.asarray(dv).reshape(-1)
    dx = np.asarray(dx).reshape(-1)
    fm = float(np.float32(M))
    for i in range(ptcl):
        b = int(dx[i] * fm)
        for j in range(r):
            dw[r * b + j] += dv[r * i + j]
    if (M // RM) > 1:
        bloks = int(math.ceil(M / RM))
        nblk = (M // bloks) + 1
        sums = []
        for k in range(nblk):
            if k * bloks >= M:
                sums.append(None)
                continue
            bb = [[dw[r * (k * bloks + t) + j] if k * bloks + t < M else 0.0 for j in range(r)]
                  for t in range(bloks)]
            s = bloks // 2
            while s > 0:
                for t in range(s):
                    for j in range(r):
                        bb[t][j] = bb[t][j] + bb[t + s][j]
                s >>= 1
            sums.append(bb[0])
        for k, sm in enumerate(sums):
            if sm is not None:
                for j in range(r):
                    dw[r * k + j] = sm[j]


# --------------------------------------------------------------------------------------
# loader
# --------------------------------------------------------------------------------------

_LOADED = {}


def load_variant(variant="1bin"):
    """Import the reference's ``<variant>/boltzmann.py`` and its kernels under the shims.

    Returns a namespace with the reference's ``BoltzmannDSMC`` class and kernel modules.
    Different variants share module names (``kernels.*``), so the module cache is
    swapped per variant.
    """
    if variant in _LOADED:
        mods = _LOADED[variant]
        sys.modules.update(mods["modules"])
        return mods["ns"]
    vdir = os.path.join(REFERENCE_ROOT, variant)
    if not os.path.isdir(vdir):
        raise FileNotFoundError(f"reference variant not found: {vdir}")
    # drop any previously imported variant's modules
    for name in list(sys.modules):
        if name == "kernels" or name.startswith("kernels.") or name == "boltzmann":
            del sys.modules[name]
    cp, rnd, cpcuda, runtime = _make_cupy()
    numba, ncuda = _make_numba()
    sys.modules["cupy"] = cp
    sys.modules["cupy.random"] = rnd
    sys.modules["cupy.cuda"] = cpcuda
    sys.modules["cupy.cuda.runtime"] = runtime
    sys.modules["numba"] = numba
    sys.modules["numba.cuda"] = ncuda
    fake_red = types.ModuleType("kernels.reduction.cuda_reduction.cuda_red")
    fake_red.calls = _cuda_red_calls
    sys.modules["kernels.reduction.cuda_reduction.cuda_red"] = fake_red
    sys.path.insert(0, vdir)
    try:
        boltz = importlib.import_module("boltzmann")
        ek = importlib.import_module("kernels.electron_kernel_numba")
        bp = importlib.import_module("kernels.bin_particles")
        pp = importlib.import_module("kernels.post_processing_1D")
        ef = importlib.import_module("kernels.EF_kernel_1D")
        hv = importlib.import_module("kernels.heavies_kernel_1D")
        red = importlib.import_module("kernels.reduction")
        red.init_reduction(False)  # what BoltzmannDSMC._init_kernels does (boltzmann.py:770)
    finally:
        sys.path.remove(vdir)
    ns = types.SimpleNamespace(
        BoltzmannDSMC=boltz.BoltzmannDSMC, boltzmann=boltz, electron=ek, bins=bp,
        post=pp, ef=ef, heavies=hv, reduction=red, cupy=cp, numba=numba,
    )
    modules = {k: v for k, v in sys.modules.items()
               if k in ("boltzmann", "kernels", "cupy", "numba") or k.startswith(("kernels.", "cupy.", "numba."))}
    _LOADED[variant] = {"ns": ns, "modules": modules}
    return ns


def as_cp(a):
    """Wrap a numpy array as a shim cupy array (aliasing, no copy)."""
    return _cp(a)

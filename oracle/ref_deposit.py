"""The reference's own GPU deposit kernels, run unchanged on the GB300 (test
infrastructure: a GPU-side checker and a measured baseline, never part of the product).

The reference deposits the particle moments with two CUDA kernels of
kernels/reduction/cuda_reduction/kernels-new.cu: ``reda`` (one float64 global atomic per
particle and moment into bnf*(N+1) fine bins, kernels-new.cu:56-73) and ``redcheck`` (sums
each node's bnf fine bins in shared memory, kernels-new.cu:8-53), launched by ``calls``
(kernels-new.cu:76-132) from post_processing (post_processing_1D.py:44-57 via
reduction/__init__.py:12-16).

``build()`` compiles that file, where it lies in the reference tree, for sm_103a into
``oracle/_ref/kernels_new.sm_103a.cubin`` (device code only; its pybind11 wrapper is not
used), when the reference tree is present; the cubin is kept with the repository copy, so
machines without the reference sources run it too. ``ReferenceDeposit`` loads it into the current CUDA context through the driver API
(ctypes on libcuda) and launches the two kernels exactly as ``calls`` does, on float64
device buffers in the reference's layout: v [ptcl][4] (w, w*ionflag, w*0, w*energy) and the
normalised positions (x + dx/2)/(L + dx).

``python -m oracle.ref_deposit`` times it against libbz's deposit on the same particles.
"""
from __future__ import annotations

import ctypes
import json
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
CUBIN = os.path.join(REF_DIR, "kernels_new.sm_103a.cubin")
REF_ROOT = os.environ.get("BZ_REFERENCE_ROOT", "/root/reference")
REF_SRC = os.path.join(REF_ROOT, "1bin", "kernels", "reduction", "cuda_reduction", "kernels-new.cu")
# the kernels' C++ names (Itanium ABI): reda(double*, double*, double*, int, int, int),
# redcheck(double*, int, int, int)
REDA = b"_Z4redaPdS_S_iii"
REDCHECK = b"_Z8redcheckPdiii"


def build(force=False):
    """Compile the reference's deposit kernels into a cubin (only where the reference tree
    is present). Returns the cubin path or None."""
    if not os.path.exists(REF_SRC):
        return CUBIN if os.path.exists(CUBIN) else None
    if os.path.exists(CUBIN) and not force and os.path.getmtime(CUBIN) >= os.path.getmtime(REF_SRC):
        return CUBIN
    os.makedirs(REF_DIR, exist_ok=True)
    import sysconfig
    try:
        import pybind11
        pyb = pybind11.get_include()
    except ImportError:
        return None
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    tmp = CUBIN + f".tmp{os.getpid()}"
    cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", f"-I{pyb}",
           f"-I{sysconfig.get_paths()['include']}", "-o", tmp, REF_SRC]
    subprocess.check_call(cmd)
    os.replace(tmp, CUBIN)
    return CUBIN


class ReferenceDeposit:
    """reda + redcheck from the cubin, launched like kernels-new.cu:76-132."""

    def __init__(self, path=CUBIN):
        if not os.path.exists(path):
            raise FileNotFoundError(f"{path} is missing (built by oracle.ref_deposit.build where the reference is)")
        import torch
        torch.cuda.init()
        torch.zeros(1, device="cuda")  # the runtime's primary context is current on this thread
        self.cu = ctypes.CDLL("libcuda.so.1")
        self.mod = ctypes.c_void_p()
        self._check(self.cu.cuModuleLoad(ctypes.byref(self.mod), path.encode()), "cuModuleLoad")
        self.reda = ctypes.c_void_p()
        self.redcheck = ctypes.c_void_p()
        self._check(self.cu.cuModuleGetFunction(ctypes.byref(self.reda), self.mod, REDA), "reda")
        self._check(self.cu.cuModuleGetFunction(ctypes.byref(self.redcheck), self.mod, REDCHECK), "redcheck")
        self.cu.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 6 + [
            ctypes.c_uint, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"CUDA driver call {what} failed: {rc}")

    def _launch(self, f, grid, block, smem, args):
        import torch
        vals = []
        for a in args:
            vals.append(ctypes.c_void_p(a.data_ptr()) if hasattr(a, "data_ptr") else ctypes.c_int(int(a)))
        ptrs = (ctypes.c_void_p * len(vals))(*[ctypes.cast(ctypes.byref(v), ctypes.c_void_p) for v in vals])
        st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
        self._check(self.cu.cuLaunchKernel(f, grid[0], grid[1], grid[2], block[0], block[1], block[2], smem, st,
                                           ptrs, None), "cuLaunchKernel")

    def calls(self, r, M, RM, dw, dv, dx, ptcl):
        """kernels-new.cu:76-132 with p unused: dw [M][r] (zeroed by the caller, as
        post_processing does), dv [ptcl][r], dx [ptcl] float64 device tensors."""
        blockx, blocky = 256, r
        self._launch(self.reda, (ptcl // blockx + 1, r // blocky + 1, 1), (blockx, blocky, 1), 0,
                     (dw, dv, dx, r, ptcl, M))
        bloks = -(-M // RM)
        if M // RM > 1:
            self._launch(self.redcheck, (M // bloks + 1, 1, 1), (bloks, 1, 1), bloks * r * 8, (dw, r, RM, M))


def reference_moments(dep, x, vx, vy, vz, w, N, L, bnf):
    """The reference's node moments [4][N+1] (ne, ni_src, ns_src, nrg) for float64 device
    tensors of the particles (ionflag 0), through its own kernels."""
    import torch
    dxg = L / N
    efac = 0.5 * (9.10938 * 1e-31) * (6.241509 * 1e18)
    n = x.numel()
    v = torch.zeros(n, 4, dtype=torch.float64, device=x.device)
    v[:, 0] = w
    v[:, 3] = w * efac * (vx * vx + vy * vy + vz * vz)
    # true division, as the reference's CuPy expression (post_processing_1D.py:44) computes
    # it: torch divides by a Python scalar through its reciprocal, which moves particles
    # that sit exactly on a node boundary
    xn = (x + 0.5 * dxg) / torch.full_like(x, L + dxg)
    M = bnf * (N + 1)
    dw = torch.zeros(M, 4, dtype=torch.float64, device=x.device)
    dep.calls(4, M, N + 1, dw, v.contiguous(), xn.contiguous(), n)
    return dw[:N + 1].t().contiguous()


def main():
    """Time the reference's deposit and libbz's on the same particles (uniform positions,
    1 eV Maxwellian, 2e7 electrons, 1024 cells, bnf 4) and print one JSON line."""
    import math

    import torch
    sys.path.insert(0, os.path.dirname(HERE))
    from boltzmann_gb300 import kernels as K

    n = int(float(sys.argv[1])) if len(sys.argv) > 1 else 20_000_000
    N, L, bnf = 1024, 2.54, 4
    g = torch.Generator(device="cuda")
    g.manual_seed(0)
    x = (torch.rand(n, generator=g, device="cuda", dtype=torch.float64) * L).float().double()
    vv = (torch.randn(n, 3, generator=g, device="cuda", dtype=torch.float64) * math.sqrt(1.5 * 1.17255e11)).float().double()
    w = torch.full((n,), 1e3, dtype=torch.float64, device="cuda")
    dep = ReferenceDeposit()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
    for _ in range(2):
        ref = reference_moments(dep, x, vv[:, 0], vv[:, 1], vv[:, 2], w, N, L, bnf)
    torch.cuda.synchronize()
    ev[0].record()
    reps = 5
    for _ in range(reps):
        ref = reference_moments(dep, x, vv[:, 0], vv[:, 1], vv[:, 2], w, N, L, bnf)
    ev[1].record()
    torch.cuda.synchronize()
    ms_ref = ev[0].elapsed_time(ev[1]) / reps
    seg = K.SegmentSet(-(-2 * n // 4096), 2048, torch.float32)
    seg.load(x.cpu().numpy(), vv[:, 0].cpu().numpy(), vv[:, 1].cpu().numpy(), vv[:, 2].cpu().numpy(),
             w.cpu().numpy())
    p = K.make_params(n_faces=N, n_nodes=N + 1, bnf=bnf, advect=1, L=L, dx=L / N, dt=1e-12, nn=3.22e22)
    mom = torch.zeros(4, N + 1, dtype=torch.float64, device="cuda")
    for _ in range(2):
        mom.zero_()
        K.seg_deposit(p, seg, mom)
    ev[2].record()
    for _ in range(reps):
        mom.zero_()
        K.seg_deposit(p, seg, mom)
    ev[3].record()
    torch.cuda.synchronize()
    ms_ours = ev[2].elapsed_time(ev[3]) / reps
    rel = [float(((mom[j] - ref[j]).abs() / ref[j].abs().clamp_min(1e-300)).max().item()) for j in (0, 3)]
    worst = int((mom[0] - ref[0]).abs().argmax().item())
    print(json.dumps({"particles": n, "cells": N, "bnf": bnf, "reference_reda_redcheck_ms": ms_ref,
                      "ours_seg_deposit_ms": ms_ours, "speedup": ms_ref / ms_ours,
                      "max_rel_diff_per_node": {"ne": rel[0], "nrg": rel[1]}, "worst_ne_node": worst,
                      "worst_ne": [float(mom[0, worst]), float(ref[0, worst])],
                      "note": "reference: float64 inputs it builds on the GPU (v[ptcl][4], normalised x) "
                              "included; ours: float32 SoA segments"}))


if __name__ == "__main__":
    main()

"""Device buffers and thin wrappers over the libbz entry points.

PyTorch is used only to own device memory and to supply the current CUDA stream;
every computation is a libbz kernel. Function names follow the reference's kernel
modules (electron_kernel, bin_particles, post_processing / reduction, EF_kernel,
heavies_kernel_fluid); argument meaning follows ``include/bz.h``.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import BzParams, Particles, Segments, call


def _ptr(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class ParticleSet:
    """Structure-of-arrays particle state (x, vx, vy, vz, w) of fixed capacity on one
    GPU, plus an int32 count word array: cnt[0] survivors, cnt[1] children, cnt[2] n."""

    FIELDS = ("x", "vx", "vy", "vz", "w")

    def __init__(self, capacity, dtype=torch.float32, device="cuda"):
        self.capacity = int(capacity)
        self.dtype = dtype
        # one allocation, 5 arrays, each 256-byte aligned
        esz = torch.finfo(dtype).bits // 8
        stride = ((self.capacity * esz + 255) // 256) * 256 // esz
        self._buf = torch.zeros(5 * stride, dtype=dtype, device=device)
        for k, f in enumerate(self.FIELDS):
            setattr(self, f, self._buf[k * stride: k * stride + self.capacity])
        self.cnt = torch.zeros(4, dtype=torch.int32, device=device)

    @property
    def suffix(self):
        return "f32" if self.dtype == torch.float32 else "f64"

    def struct(self):
        return Particles(*(getattr(self, f).data_ptr() for f in self.FIELDS))

    def n_ptr(self):
        return ctypes.c_void_p(self.cnt.data_ptr() + 8)

    def counts_ptr(self):
        return ctypes.c_void_p(self.cnt.data_ptr())

    def n(self):
        """Particle count (reads device memory: a synchronisation)."""
        return int(self.cnt[2].item())

    def load(self, x, vx, vy, vz, w):
        n = len(x)
        if n > self.capacity:
            raise ValueError(f"{n} particles exceed capacity {self.capacity}")
        for f, a in zip(self.FIELDS, (x, vx, vy, vz, w)):
            getattr(self, f)[:n].copy_(torch.as_tensor(np.asarray(a), dtype=self.dtype))
        self.cnt.zero_()
        self.cnt[2] = n
        self.cnt[0] = n

    def to_numpy(self, n=None):
        n = self.n() if n is None else n
        return {f: getattr(self, f)[:n].detach().cpu().numpy().astype(np.float64) for f in self.FIELDS}


class SegmentSet:
    """Segmented particle state (include/bz.h, bz_segments_*): nseg segments of 2*half
    slots; segment s holds run 0 at [s*2h, s*2h+counts[2s]) and run 1 at
    [s*2h+h, s*2h+h+counts[2s+1]). The solver's hot loop pushes these one warp per
    segment with no ordering between segments."""

    FIELDS = ParticleSet.FIELDS

    def __init__(self, nseg, half, dtype=torch.float32, device="cuda"):
        if half % 4:
            raise ValueError("half must be a multiple of 4")
        self.nseg, self.half, self.dtype = int(nseg), int(half), dtype
        self.capacity = self.nseg * 2 * self.half
        esz = torch.finfo(dtype).bits // 8
        stride = ((self.capacity * esz + 255) // 256) * 256 // esz
        self._buf = torch.zeros(5 * stride, dtype=dtype, device=device)
        for k, f in enumerate(self.FIELDS):
            setattr(self, f, self._buf[k * stride: k * stride + self.capacity])
        self.counts = torch.zeros(2 * self.nseg, dtype=torch.int32, device=device)
        self.device = device

    @property
    def suffix(self):
        return "f32" if self.dtype == torch.float32 else "f64"

    def struct(self):
        return Segments(*(getattr(self, f).data_ptr() for f in self.FIELDS), self.counts.data_ptr(), self.nseg,
                        self.half)

    def n(self):
        """Occupied slots (run 0 and run 1 of every segment)."""
        return int(self.counts.sum().item())

    def n_live(self):
        """Particles (w != 0) among the occupied slots: after an in-place resampling the runs
        may hold slots its merges emptied until the next push drops them."""
        idx = torch.as_tensor(self.slots("segments"), device=self.device)
        return int((self.w[idx] != 0).sum().item()) if idx.numel() else 0

    def load(self, x, vx, vy, vz, w, ws=None, status=None):
        """Spread a dense particle list evenly over the segments (on the device)."""
        n = len(x)
        tmp = ParticleSet(max(n, 1), self.dtype, self.device)
        tmp.load(x, vx, vy, vz, w)
        if n > self.nseg * self.half:
            raise RuntimeError(f"{n} particles exceed the {self.nseg} x {self.half} slots of run 0")
        st = status if status is not None else torch.zeros(1, dtype=torch.int32, device=self.device)
        seg_repack(None, self, st, ws or Workspace(self.device), app=tmp)
        return st

    def slots(self, order="runs"):
        """Host-side slot indices of the live particles. order='runs': run 0 of every
        segment, then run 1 of every segment (survivors in input order, then children in
        parent order after one push); order='segments': segment by segment."""
        c = self.counts.cpu().numpy().reshape(-1, 2)
        base = np.arange(self.nseg, dtype=np.int64) * 2 * self.half
        r0 = [np.arange(b, b + k) for b, k in zip(base, c[:, 0])]
        r1 = [np.arange(b + self.half, b + self.half + k) for b, k in zip(base, c[:, 1])]
        if order == "runs":
            parts = r0 + r1
        else:
            parts = [a for pair in zip(r0, r1) for a in pair]
        return np.concatenate(parts) if parts else np.zeros(0, dtype=np.int64)

    def to_numpy(self, order="runs"):
        idx = torch.as_tensor(self.slots(order), device=self.device)
        return {f: getattr(self, f)[idx].detach().cpu().numpy().astype(np.float64) for f in self.FIELDS}


class Workspace:
    """Grow-only device scratch per purpose."""

    def __init__(self, device="cuda"):
        self.device = device
        self._bufs = {}

    def get(self, name, nbytes):
        b = self._bufs.get(name)
        if b is None or b.numel() < nbytes:
            b = torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=self.device)
            self._bufs[name] = b
        return b


def make_params(*, n_faces, n_nodes, bnf, advect, L, dx, dt, nn, gas_sigma=0.0, e_exc=11.5, nu_max=0.0,
                xs_mode=_lib.XS_TABLE, coll_model=_lib.COLL_DIRECT, xs_table=None, xs_emin=0.01, xs_emax=1000.0,
                flags=0, seed=0, step=0, step_ptr=None):
    p = BzParams()
    p.n_faces, p.n_nodes, p.bnf, p.advect = int(n_faces), int(n_nodes), int(bnf), int(advect)
    p.L, p.dx, p.dt, p.nn = float(L), float(dx), float(dt), float(nn)
    p.gas_sigma, p.e_exc, p.nu_max = float(gas_sigma), float(e_exc), float(nu_max)
    p.xs_mode, p.coll_model, p.flags = int(xs_mode), int(coll_model), int(flags)
    if xs_table is not None:
        p.xs_n = int(xs_table.shape[1])
        p.xs_table = xs_table.data_ptr()
    else:
        p.xs_n = 0
        p.xs_table = None
    p.xs_emin, p.xs_emax = float(xs_emin), float(xs_emax)
    p.seed, p.step = int(seed), int(step)
    p.step_ptr = None if step_ptr is None else step_ptr.data_ptr()
    return p


# --------------------------------------------------------------------------------------
# entry points
# --------------------------------------------------------------------------------------

def electron_kernel(params, src: ParticleSet, dst: ParticleSet, E, status, ws: Workspace, moments=None,
                    replay_R=None, replay_gas=None, fast=True):
    """Push + collide src into dst (compacted, children appended); optionally deposit
    moments [4, n_nodes] (float64, accumulated). electron_kernel_numba.py:291-303 plus
    the deposit and compaction of post_processing_1D.py:40-68. ``fast``: with the larger
    workspace the push runs through the segmented kernel and a gather (same results);
    otherwise the single-pass push with the decoupled look-back."""
    if src.dtype != dst.dtype:
        raise TypeError("src and dst precision differ")
    if E.dtype != src.dtype:
        raise TypeError("E must have the particle precision")
    lib = _lib.load()
    if fast:
        nbytes = getattr(lib, f"bz_push_workspace_fast_{src.suffix}")(src.capacity, params.n_nodes)
        w = ws.get("push_fast", nbytes)
    else:
        w = ws.get("push", lib.bz_push_workspace(max(src.capacity, dst.capacity)))
    call(f"bz_push_collide_{src.suffix}", ctypes.byref(params), src.struct(), src.n_ptr(), src.capacity, dst.struct(),
         dst.capacity, dst.counts_ptr(), _ptr(E), _ptr(replay_R), _ptr(replay_gas), _ptr(moments), _ptr(w),
         w.numel(), _ptr(status), _stream())


def deposit(params, s: ParticleSet, moments, ionflag=None):
    """The moments post_processing deposits (kernels-new.cu reda/redcheck), race-free."""
    call(f"bz_deposit_{s.suffix}", ctypes.byref(params), s.struct(), s.n_ptr(), s.capacity, _ptr(ionflag),
         _ptr(moments), _stream())


def bin_particles(params, s: ParticleSet, edges, min_wt, perm, offsets, counts, hw_counts, status, ws: Workspace):
    """Cell x energy-bin stable sort (bin_particles.py:7-31 and its 3/5-bin versions)."""
    nb = int(edges.numel()) + 1
    nkeys = params.n_nodes * nb
    nbytes = _lib.load().bz_bin_workspace(s.capacity, nkeys)
    w = ws.get("bin", nbytes)
    call(f"bz_bin_{s.suffix}", ctypes.byref(params), s.struct(), s.n_ptr(), s.capacity, nb,
         _ptr(edges) if nb > 1 else None, float(min_wt), _ptr(perm), _ptr(offsets), _ptr(counts), _ptr(hw_counts),
         _ptr(w), w.numel(), _ptr(status), _stream())


def resample(params, s: ParticleSet, out: ParticleSet, nb, targets, max_ppc, min_wt, split_below, merge_at,
             merge_keep, perm, offsets, counts, hw_counts, status, ws: Workspace, need=None, replay_u=None,
             cons_diag=None):
    """ES-WPNC split / merge (boltzmann.py:799-890), appended into s, compacted into out."""
    nkeys = params.n_nodes * nb
    nbytes = _lib.load().bz_resample_workspace(s.capacity, nkeys)
    w = ws.get("resample", nbytes)
    call(f"bz_resample_{s.suffix}", ctypes.byref(params), s.struct(), s.n_ptr(), s.capacity, out.struct(),
         out.n_ptr(), nb, _ptr(targets), _ptr(max_ppc), float(min_wt), float(split_below), float(merge_at),
         float(merge_keep), _ptr(perm), _ptr(offsets), _ptr(counts), _ptr(hw_counts), _ptr(replay_u), _ptr(need),
         _ptr(cons_diag), _ptr(w), w.numel(), _ptr(status), _stream())


def compact(s: ParticleSet, out: ParticleSet, status, ws: Workspace):
    """Order-preserving removal of w == 0 particles (boltzmann.py:879-883)."""
    w = ws.get("compact", _lib.load().bz_compact_workspace(s.capacity))
    call(f"bz_compact_{s.suffix}", s.struct(), s.n_ptr(), s.capacity, out.struct(), out.capacity, out.n_ptr(), _ptr(w),
         w.numel(), _ptr(status), _stream())


# --------------------------------------------------------------------------------------
# segmented state
# --------------------------------------------------------------------------------------

def seg_electron_kernel(params, src: SegmentSet, dst: SegmentSet, E, status, seg_flags, ws: Workspace, moments=None,
                        replay_R=None, replay_gas=None, n_pushed=None):
    """Push + collide a segmented state (one warp per segment, no inter-segment order);
    n_pushed (int64 device scalar, optional) accumulates the particles pushed."""
    if src.dtype != dst.dtype or E.dtype != src.dtype:
        raise TypeError("precision mismatch")
    if n_pushed is not None and n_pushed.dtype != torch.int64:
        raise TypeError("n_pushed must be int64")
    w = ws.get("seg_push", _lib.load().bz_seg_push_workspace_nodes(params.n_nodes))
    call(f"bz_seg_push_collide_{src.suffix}", ctypes.byref(params), src.struct(), dst.struct(), _ptr(E),
         _ptr(replay_R), _ptr(replay_gas), _ptr(moments), _ptr(n_pushed), _ptr(w), w.numel(), _ptr(seg_flags),
         _ptr(status), _stream())


def seg_push_shapes():
    """CTA shapes (threads, particles per lane, CTAs per SM, prefetch) of the float32
    table + deposit segmented push; index 0 is the library default."""
    lib = _lib.load()
    out = []
    for k in range(lib.bz_seg_push_shapes()):
        t, i, m, f = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        call("bz_seg_push_shape_info", k, ctypes.byref(t), ctypes.byref(i), ctypes.byref(m), ctypes.byref(f))
        out.append((t.value, i.value, m.value, bool(f.value)))
    return out


def select_seg_push_shape(k):
    call("bz_seg_push_select", int(k))


def autotune_seg_push(params, src: SegmentSet, dst: SegmentSet, E, status, seg_flags, ws: Workspace, moments,
                      reps=10, warmup=2):
    """Time every CTA shape of the float32 table + deposit push on src -> dst with CUDA
    events and select the fastest (process-wide, for later launches and captures). src
    is only read; dst, moments and the flag words are left as before the call. Returns
    (selected index, per-shape milliseconds)."""
    shapes = seg_push_shapes()
    if src.dtype != torch.float32 or len(shapes) < 2:
        return _lib.load().bz_seg_push_selected(), []
    saved = (status.clone(), seg_flags.clone(), moments.clone(), dst.counts.clone())
    st = torch.cuda.current_stream()
    times = []
    for k in range(len(shapes)):
        select_seg_push_shape(k)
        for _ in range(warmup):
            seg_electron_kernel(params, src, dst, E, status, seg_flags, ws, moments=moments)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            seg_electron_kernel(params, src, dst, E, status, seg_flags, ws, moments=moments)
        e1.record(st)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / reps)
    # the default (shape 0) stays unless another shape is clearly faster: the ranking of
    # close shapes moves with the state (collision rate), the default is the best measured
    # on a heated CCP
    best = int(np.argmin(times))
    if times[best] > 0.97 * times[0]:
        best = 0
    select_seg_push_shape(best)
    status.copy_(saved[0]); seg_flags.copy_(saved[1]); moments.copy_(saved[2]); dst.counts.copy_(saved[3])
    return best, times


def seg_repack(src, dst: SegmentSet, status, ws: Workspace, app: ParticleSet = None, app_n=None, only_if=None,
               clear=None, name="seg_repack"):
    """Particles with w != 0 of src (may be None), then app[0:n), spread over dst."""
    nseg_in = src.nseg if src is not None else 0
    w = ws.get(name, _lib.load().bz_seg_repack_workspace(nseg_in))
    suffix = dst.suffix
    ins = ctypes.byref(src.struct()) if src is not None else None
    if app is not None:
        ap, an, acap = app.struct(), (app_n if app_n is not None else app.n_ptr()), app.capacity
    else:
        ap, an, acap = Particles(), None, 0
    call(f"bz_seg_repack_{suffix}", ins, ap, an, acap, dst.struct(), _ptr(w), w.numel(), _ptr(only_if), _ptr(clear),
         _ptr(status), _stream())


def seg_rebalance(s: SegmentSet, scratch: SegmentSet, status, ws: Workspace, only_if=None, clear=None,
                  name="seg_rebalance"):
    """Spread s's live particles evenly over its segments again (through scratch), in one
    launch; skipped unless only_if's BZ_SEG_NEEDS_REPACK bit is set (when given)."""
    w = ws.get(name, _lib.load().bz_seg_repack_workspace(s.nseg))
    call(f"bz_seg_rebalance_{s.suffix}", s.struct(), scratch.struct(), _ptr(w), w.numel(), _ptr(only_if), _ptr(clear),
         _ptr(status), _stream())


def seg_place(s: SegmentSet, app: ParticleSet, scratch: SegmentSet, status, ws: Workspace, app_n=None, clear=None,
              name="seg_place"):
    """app[0:n) into the free slots of s's segments, in place (through scratch and back
    into s when they do not fit that way)."""
    w = ws.get(name, _lib.load().bz_seg_place_workspace(s.nseg))
    an = _ptr(app_n) if app_n is not None else app.n_ptr()
    call(f"bz_seg_place_{s.suffix}", s.struct(), app.struct(), an, app.capacity, scratch.struct(), _ptr(w),
         w.numel(), _ptr(clear), _ptr(status), _stream())


def seg_deposit(params, s: SegmentSet, moments):
    call(f"bz_seg_deposit_{s.suffix}", ctypes.byref(params), s.struct(), _ptr(moments), _stream())


def seg_eedf(params, s: SegmentSet, hist, emin, emax):
    """Add sum(w) per (deposit node, log energy bin) to hist [n_nodes, nbins] (float64)."""
    call(f"bz_seg_eedf_{s.suffix}", ctypes.byref(params), s.struct(), int(hist.shape[1]), float(emin), float(emax),
         _ptr(hist), _stream())


def seg_bin_particles(params, s: SegmentSet, edges, min_wt, perm, offsets, counts, hw_counts, status, ws: Workspace,
                      check=None):
    """Bin s by (cell, energy bin). ``check`` = (targets, split_below, merge_at, need): the
    resampling trigger is evaluated from the counts first (need gets 1 or 0) and the sort
    runs only when it is 1 (perm and offsets are then valid only in that case)."""
    nb = int(edges.numel()) + 1
    w = ws.get("seg_bin", _lib.load().bz_seg_bin_workspace(s.nseg, s.capacity))
    if check is None:
        call(f"bz_seg_bin_{s.suffix}", ctypes.byref(params), s.struct(), nb, _ptr(edges) if nb > 1 else None,
             float(min_wt), _ptr(perm), _ptr(offsets), _ptr(counts), _ptr(hw_counts), _ptr(w), w.numel(),
             _ptr(status), _stream())
        return
    targets, split_below, merge_at, need = check
    call(f"bz_seg_bin_check_{s.suffix}", ctypes.byref(params), s.struct(), nb, _ptr(edges) if nb > 1 else None,
         float(min_wt), _ptr(perm), _ptr(offsets), _ptr(counts), _ptr(hw_counts), _ptr(targets), float(split_below),
         float(merge_at), _ptr(need), _ptr(w), w.numel(), _ptr(status), _stream())


def seg_resample(params, s: SegmentSet, app: ParticleSet, out: SegmentSet, nb, targets, max_ppc, min_wt, split_below,
                 merge_at, merge_keep, perm, offsets, counts, hw_counts, status, seg_flags, ws: Workspace, need=None,
                 replay_u=None, cons_diag=None, in_place=False):
    """ES-WPNC resampling of s: the result in out, or with ``in_place`` in s itself (out is
    then the scratch of a repack, needed only when the appended particles do not fit)."""
    if in_place:
        params = type(params).from_buffer_copy(params)
        params.flags |= _lib.RESAMPLE_IN_PLACE
    nkeys = params.n_nodes * nb
    w = ws.get("seg_resample", _lib.load().bz_seg_resample_workspace(s.nseg, s.capacity, nkeys))
    call(f"bz_seg_resample_{s.suffix}", ctypes.byref(params), s.struct(), app.struct(), app.capacity, out.struct(), nb,
         _ptr(targets), _ptr(max_ppc), float(min_wt), float(split_below), float(merge_at), float(merge_keep),
         _ptr(perm), _ptr(offsets), _ptr(counts), _ptr(hw_counts), _ptr(replay_u), _ptr(need), _ptr(cons_diag),
         _ptr(w), w.numel(), _ptr(seg_flags), _ptr(status), _stream())


def grid_update(n_nodes, moments, ni, Te, g2):
    call("bz_grid_update", int(n_nodes), _ptr(moments), _ptr(ni), _ptr(Te), _ptr(g2), _stream())


def ion_source_closure(n_nodes, rate, moments):
    """moments[1] = rate * moments[0] per node (the ion source from a rate closure)."""
    call("bz_ion_source_closure", int(n_nodes), _ptr(rate), _ptr(moments), _stream())


def heavies_kernel_fluid(N, dx, dt, mu_i, D_i, E, ni, Ji, brk=None):
    call("bz_ion_fluid", int(N), float(dx), float(dt), float(mu_i), float(D_i), _ptr(E), _ptr(ni), _ptr(Ji),
         _ptr(brk), _stream())


def poisson_factor(N, dx, diag, lower, plan):
    """Banded Cholesky factor (diag, lower: N-1 each) and the solve plan (4*(N-1))."""
    call("bz_poisson_factor", int(N), float(dx), _ptr(diag), _ptr(lower), _ptr(plan))


def EF_kernel(N, dx, eps0, V0, freq, t, ne, ni, plan, V, E, E32=None, t_dev=None):
    call("bz_poisson", int(N), float(dx), float(eps0), float(V0), float(freq), float(t), _ptr(t_dev), _ptr(ne),
         _ptr(ni), _ptr(plan), _ptr(V), _ptr(E), _ptr(E32), _stream())


def field_step(N, dx, dt, mu_i, D_i, eps0, V0, freq, moments, ni, Te, g2, t_dev, step_dev, plan, V, E, E32, Ji,
               brk=None):
    """Grid update, clock, ion fluid and Poisson of one step in one launch."""
    call("bz_field_step", int(N), float(dx), float(dt), float(mu_i), float(D_i), float(eps0), float(V0), float(freq),
         _ptr(moments), _ptr(ni), _ptr(Te), _ptr(g2), _ptr(t_dev), _ptr(step_dev), _ptr(plan), _ptr(V), _ptr(E),
         _ptr(E32), _ptr(Ji), _ptr(brk), _stream())


def field_step_coop(N, dx, dt, mu_i, D_i, eps0, V0, freq, moments, ni, Te, g2, t_dev, step_dev, plan, V, E, E32, Ji,
                    brk=None, ws: "Workspace" = None):
    """field_step spread over ceil((N-1)/64) CTAs: one thread-block cluster where it fits,
    else one cooperative launch."""
    w = (ws or Workspace(moments.device)).get("field_coop", _lib.load().bz_field_step_coop_workspace(int(N)))
    call("bz_field_step_coop", int(N), float(dx), float(dt), float(mu_i), float(D_i), float(eps0), float(V0),
         float(freq), _ptr(moments), _ptr(ni), _ptr(Te), _ptr(g2), _ptr(t_dev), _ptr(step_dev), _ptr(plan), _ptr(V),
         _ptr(E), _ptr(E32), _ptr(Ji), _ptr(brk), _ptr(w), w.numel(), _stream())


def philox(ctr, key, variant=0):
    """Philox4x32-10 on the device: ctr [n, 4] and key [n, 2] int64 tensors holding uint32
    values (or numpy arrays); returns [n, 4] int64 (uint32 values)."""
    c = torch.as_tensor(np.asarray(ctr, dtype=np.uint32).view(np.int32), device="cuda").contiguous()
    k = torch.as_tensor(np.asarray(key, dtype=np.uint32).view(np.int32), device="cuda").contiguous()
    n = c.shape[0]
    out = torch.zeros(n, 4, dtype=torch.int32, device="cuda")
    call("bz_philox4x32_10", _ptr(c), _ptr(k), int(n), int(variant), _ptr(out), _stream())
    return out.cpu().numpy().view(np.uint32).astype(np.int64)


def field_step_select(mode):
    """Form of field_step_coop: 0 cluster where it fits (default), 1 cooperative, 2 cluster."""
    call("bz_field_step_select", int(mode))


def field_step_selected():
    return int(_lib.load().bz_field_step_selected())


def advance_clock(t_dev, step_dev, dt):
    call("bz_advance_clock", _ptr(t_dev), _ptr(step_dev), float(dt), _stream())


# ------------------------------------------------------------------------------------ surrogate network
def seg_sample_energy(params, s: SegmentSet, cdf, emin, emax, seed, scale=None):
    """Velocities of every live particle drawn from cdf [n_keys, nbins] (float64, cumulative
    weight fractions of log bins over [emin, emax) eV) of its key (deposit node / swarm);
    the energies times scale[key] when given."""
    call(f"bz_seg_sample_energy_{s.suffix}", ctypes.byref(params), s.struct(), int(cdf.shape[0]), int(cdf.shape[1]),
         float(emin), float(emax), _ptr(cdf), _ptr(scale), int(seed), _stream())


def mlp_sync(prm, wb, wt):
    call("bz_mlp_sync", _ptr(prm), _ptr(wb), _ptr(wt), _stream())


def mlp_forward(wb, prm, x, y, idx=None, z=None):
    call("bz_mlp_forward", _ptr(wb), _ptr(prm), _ptr(x), _ptr(idx), int(y.shape[0]), _ptr(y), _ptr(z), _stream())


def mlp_backward(wb, wt, prm, x, t, wcol, y, z, grad, loss, idx=None, ws: "Workspace" = None):
    """Loss and its gradient (added to grad). With a workspace the tcgen05 backward runs
    (deterministic per-CTA partial sums); without one the mma.sync backward (atomics)."""
    n = int(y.shape[0])
    w = None if ws is None else ws.get("mlp_bwd", _lib.load().bz_mlp_backward_workspace(n))
    call("bz_mlp_backward", _ptr(wb), _ptr(wt), _ptr(prm), _ptr(x), _ptr(t), _ptr(wcol), _ptr(idx), n, _ptr(y),
         _ptr(z), _ptr(grad), _ptr(loss), _ptr(w), 0 if w is None else w.numel(), _stream())


def mlp_adam(prm, grad, m, v, wb, wt, step, lr, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0):
    call("bz_mlp_adam", _ptr(prm), _ptr(grad), _ptr(m), _ptr(v), _ptr(wb), _ptr(wt), int(step), float(lr),
         float(beta1), float(beta2), float(eps), float(weight_decay), _stream())


def mlp_batch(n_rows, idx, seed, step):
    call("bz_mlp_batch", int(n_rows), int(idx.numel()), int(seed), int(step), _ptr(idx), _stream())


def mlp_train_step(prm, grad, m, v, wb, wt, x, t, wcol, batch, seed, step, lr, loss, ws: Workspace, beta1=0.9,
                   beta2=0.999, eps=1e-8, weight_decay=0.0):
    w = ws.get("mlp_train", _lib.load().bz_mlp_train_workspace(int(batch)))
    call("bz_mlp_train_step", _ptr(prm), _ptr(grad), _ptr(m), _ptr(v), _ptr(wb), _ptr(wt), _ptr(x), _ptr(t),
         _ptr(wcol), int(x.shape[0]), int(batch), int(seed), int(step), float(lr), float(beta1), float(beta2),
         float(eps), float(weight_decay), _ptr(loss), _ptr(w), w.numel(), _stream())

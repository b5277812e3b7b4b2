"""Host-side mirror of the reference's estimate-and-mark interface.

Method names and argument meaning follow the PUMI calls they replace
(spr/spr.h:33-62, ma/maSize.h:30-113, ma/maRefine.cc:395,
ma/maCoarsen.cc:287, ma/maShape.h:24-26); apf fields become numpy arrays
in MDS index order.  Errors raise :class:`SprgError` where the reference
would abort.
"""
import ctypes
import json

import numpy as np

from . import _lib
from ._lib import SprgError, check  # noqa: F401


def _f64(a, shape=None):
    a = np.ascontiguousarray(a, dtype=np.float64)
    if shape is not None and a.shape != shape:
        a = a.reshape(shape)
    return a


class Context:
    """A mesh flattened onto one GPU (sprg_create)."""

    def __init__(self, mesh, device=0, precision="fp64"):
        self._lib = _lib.load()
        self.mesh = mesh
        self._view = mesh.view()
        h = ctypes.c_void_p()
        rc = self._lib.sprg_create(ctypes.byref(self._view), device, ctypes.byref(h))
        if rc:
            raise SprgError(rc, "sprg_create failed")
        self.h = h
        self.set_precision(precision)

    # -- lifetime -------------------------------------------------------
    def close(self):
        if getattr(self, "h", None):
            self._lib.sprg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        check(rc, self.h)

    def set_precision(self, precision):
        code = {"fp64": _lib.SPRG_FP64, "fp32": _lib.SPRG_FP32, "learned": _lib.SPRG_LEARNED}[precision]
        self._check(self._lib.sprg_set_precision(self.h, code))
        self.precision = precision
        if precision == "learned" and not getattr(self, "_mlp_set", False):
            from . import learned
            self.set_mlp_params(learned.default_params())

    # ---- learned form ----------------------------------------------------
    def set_mlp_params(self, params):
        """FP32 parameter vector (W1, b1, W2, b2, W3, b3; see learned.py)."""
        p = np.ascontiguousarray(params, dtype=np.float32)
        if p.size != _lib.MLP_PARAMS:
            raise ValueError(f"expected {_lib.MLP_PARAMS} parameters, got {p.size}")
        self._check(self._lib.sprg_set_mlp_params(self.h, p.ctypes.data, p.size))
        self._mlp_set = True

    def set_learned_options(self, use_mlp=True, z_max=8.0):
        self._check(self._lib.sprg_set_learned_options(self.h, 1 if use_mlp else 0, float(z_max)))

    def learned_features(self, d_u, d_x, d_aux):
        """Network inputs for a device field (V doubles): d_x [V][128] BF16,
        d_aux [V][5] FP32 (device pointers)."""
        self._check(self._lib.sprg_learned_features(self.h, d_u, d_x, d_aux))

    def set_stream(self, stream_handle):
        self._check(self._lib.sprg_set_stream(self.h, ctypes.c_void_p(stream_handle)))

    def profile(self, on=True):
        """Per-kernel CUDA-event timing on the context stream."""
        self._check(self._lib.sprg_profile_enable(self.h, 1 if on else 0))

    def profile_report(self, reset=True):
        """{kernel: (launches, total_ms)} since the last reset."""
        import json
        raw = json.loads(self._lib.sprg_profile_report(self.h, 1 if reset else 0).decode())
        return {k: (int(v[0]), float(v[1])) for k, v in raw.items()}

    def debug_read(self, name, dtype, count):
        """Copy of a named internal device buffer (instrumentation)."""
        out = np.empty(count, dtype)
        self._check(self._lib.sprg_debug_read(self.h, name.encode(), out.ctypes.data, out.nbytes))
        return out

    def test_hooks(self, wait_polls=0, alloc_fail_after=-1):
        """Failure-path hooks (sprg_test_hooks): a network-kernel wait limit
        in polls, and a device allocation that fails after n more."""
        self._check(self._lib.sprg_test_hooks(self.h, int(wait_polls), int(alloc_fail_after)))

    def e2e_timing(self, on=True):
        """Stage timing of estimate_and_mark calls (clears the sums)."""
        self._check(self._lib.sprg_e2e_timing(self.h, 1 if on else 0))

    def e2e_timing_report(self):
        """Per-call averages (ms) of the stages of the timed calls."""
        return json.loads(self._lib.sprg_e2e_timing_report(self.h).decode())

    @property
    def last_launch_count(self):
        return int(self._lib.sprg_last_launch_count(self.h))

    # -- spr ------------------------------------------------------------
    def getGradIPField(self, f, name="grad", order=1):
        """spr::getGradIPField: SCALAR (V,) -> (T,3); VECTOR (V,3) -> (T,9)."""
        f = _f64(f)
        ncin = 1 if f.ndim == 1 else f.shape[1]
        out = np.empty((self.mesh.n_elems, 3 * ncin), np.float64)
        self._check(self._lib.sprg_get_grad_ip_field(self.h, f.ctypes.data, ncin, order, out.ctypes.data))
        return out

    def recoverField(self, ip):
        """spr::recoverField: (T,nc) integration-point field -> (V,nc) nodal field."""
        ip = _f64(ip)
        nc = ip.shape[1]
        out = np.empty((self.mesh.n_verts, nc), np.float64)
        self._check(self._lib.sprg_recover_field(self.h, ip.ctypes.data, nc, out.ctypes.data))
        return out

    def getSPRSizeField(self, ip, adapt_ratio):
        """spr::getSPRSizeField: returns (size (V,), info dict)."""
        ip = _f64(ip)
        out = np.empty(self.mesh.n_verts, np.float64)
        info = _lib.SizeInfo()
        self._check(self._lib.sprg_get_spr_size_field(self.h, ip.ctypes.data, ip.shape[1], float(adapt_ratio),
                                                      out.ctypes.data, ctypes.byref(info)))
        return out, info.as_dict()

    def getTargetSPRSizeField(self, ip, target, alpha=0.25, beta=2.0):
        """spr::getTargetSPRSizeField: returns (size (V,), info dict)."""
        ip = _f64(ip)
        out = np.empty(self.mesh.n_verts, np.float64)
        info = _lib.SizeInfo()
        self._check(self._lib.sprg_get_target_spr_size_field(self.h, ip.ctypes.data, ip.shape[1], int(target),
                                                             float(alpha), float(beta), out.ctypes.data,
                                                             ctypes.byref(info)))
        return out, info.as_dict()

    # -- ma -------------------------------------------------------------
    def makeSizeField(self, size=None, sizes=None, frames=None, logInterpolation=False):
        """ma::makeSizeField(m, size) or ma::makeSizeField(m, sizes, frames, logInterpolation)."""
        return SizeField(self, size, sizes, frames, logInterpolation)

    def measure_edges(self, size=None):
        out = np.empty(self.mesh.n_edges, np.float64)
        p = None if size is None else _f64(size)
        self._check(self._lib.sprg_measure_edges(self.h, None if p is None else p.ctypes.data, out.ctypes.data))
        return out

    def measure_edges_aniso(self, sizes, frames):
        sizes = _f64(sizes)
        frames = _f64(frames).reshape(self.mesh.n_verts, 9)
        out = np.empty(self.mesh.n_edges, np.float64)
        self._check(self._lib.sprg_measure_edges_aniso(self.h, sizes.ctypes.data, frames.ctypes.data,
                                                       out.ctypes.data))
        return out

    def measure_edges_log_aniso(self, sizes, frames):
        """makeSizeField(m, sizes, frames, true) (LogAnisoSizeField) + measure."""
        sizes = _f64(sizes)
        frames = _f64(frames).reshape(self.mesh.n_verts, 9)
        out = np.empty(self.mesh.n_edges, np.float64)
        self._check(self._lib.sprg_measure_edges_log_aniso(self.h, sizes.ctypes.data, frames.ctypes.data,
                                                           out.ctypes.data))
        return out

    def measureQualityLog(self, sizes, frames):
        """measureTetQuality / measureTriQuality under the LogAnisoSizeField."""
        sizes = _f64(sizes)
        frames = _f64(frames).reshape(self.mesh.n_verts, 9)
        q = np.empty(self.mesh.n_elems, np.float64)
        self._check(self._lib.sprg_measure_quality_log_aniso(self.h, sizes.ctypes.data, frames.ctypes.data,
                                                             q.ctypes.data))
        return q

    def _mark(self, which, flags):
        if flags.dtype != np.int32 or not flags.flags["C_CONTIGUOUS"]:
            raise TypeError("flags must be a contiguous int32 array")
        n = ctypes.c_long()
        self._check(self._lib.sprg_mark_edges(self.h, which, flags.ctypes.data, ctypes.byref(n)))
        return n.value

    def markEdgesToSplit(self, flags):
        """ma::markEdgesToSplit on the resident edge lengths; flags updated in place."""
        return self._mark(_lib.MARK_SPLIT, flags)

    def markEdgesToCollapse(self, flags):
        """ma::markEdgesToCollapse on the resident edge lengths; flags updated in place."""
        return self._mark(_lib.MARK_COLLAPSE, flags)

    def measureQuality(self, size=None, sizes=None, frames=None):
        """measureTetQuality / measureTriQuality (useMax = true) of every element."""
        q = np.empty(self.mesh.n_elems, np.float64)
        s = None if size is None else _f64(size)
        ss = None if sizes is None else _f64(sizes)
        ff = None if frames is None else _f64(frames).reshape(self.mesh.n_verts, 9)
        self._check(self._lib.sprg_measure_quality(
            self.h, None if s is None else s.ctypes.data, None if ss is None else ss.ctypes.data,
            None if ff is None else ff.ctypes.data, q.ctypes.data))
        return q

    # -- incremental update after host topology changes -----------------
    def update_mesh(self, new_mesh, delta=None):
        """Send the rows of `new_mesh` that differ from the context's mesh
        (moved vertices, new or rewired elements and edges, the counts) and
        rebuild the device structures; the context then holds `new_mesh`.
        `delta`: those rows when the caller knows them (mesh_delta's form),
        else mesh_delta computes them.  Returns the delta's row counts
        (vertices, elements, edges)."""
        if new_mesh.dim != self.mesh.dim:
            raise ValueError("the dimension cannot change")
        d = mesh_delta(self.mesh, new_mesh) if delta is None else delta
        keep = []  # arrays referenced by the ctypes struct stay alive for the call

        def ptr(a):
            if a is None:
                return None
            keep.append(a)
            return a.ctypes.data
        off = getattr(new_mesh, "v2e_off", None)
        el = getattr(new_mesh, "v2e", None)
        off = None if off is None else np.ascontiguousarray(off, np.int32)
        el = None if el is None else np.ascontiguousarray(el, np.int32)
        delta = _lib.MeshDelta(new_mesh.n_verts, new_mesh.n_elems, new_mesh.n_edges,
                               len(d["vert_ids"]), ptr(d["vert_ids"]), ptr(d["coords"]),
                               len(d["elem_ids"]), ptr(d["elem_ids"]), ptr(d["elem_verts"]),
                               len(d["edge_ids"]), ptr(d["edge_ids"]), ptr(d["edge_verts"]),
                               ptr(off), ptr(el))
        self._check(self._lib.sprg_update_mesh(self.h, ctypes.byref(delta)))
        self.mesh = new_mesh
        self._view = new_mesh.view()
        return len(d["vert_ids"]), len(d["elem_ids"]), len(d["edge_ids"])

    # -- MA sweeps around the marks -------------------------------------
    def _size_kind(self, size, sizes, frames, identity, log=False):
        if identity:
            return _lib.SIZE_IDENTITY, None, None, None
        if sizes is not None or frames is not None:
            return (_lib.SIZE_LOG_ANISO if log else _lib.SIZE_ANISO, None,
                    _f64(sizes).reshape(self.mesh.n_verts, 3), _f64(frames).reshape(self.mesh.n_verts, 9))
        return _lib.SIZE_ISO, None if size is None else _f64(size), None, None

    @staticmethod
    def _ptr(a):
        return None if a is None else a.ctypes.data

    def measure_vertex_pairs(self, pairs, size=None, sizes=None, frames=None, identity=False, log=False):
        """SizeField::measure of the would-be edges (vertex pairs, n x 2);
        log=True selects the log-interpolated anisotropic field."""
        kind, s, ss, ff = self._size_kind(size, sizes, frames, identity, log)
        pr = np.ascontiguousarray(pairs, np.int32).reshape(-1, 2)
        out = np.empty(pr.shape[0], np.float64)
        self._check(self._lib.sprg_measure_vertex_pairs(self.h, kind, self._ptr(s), self._ptr(ss), self._ptr(ff),
                                                        pr.shape[0], pr.ctypes.data, out.ctypes.data))
        return out

    def getMaximumEdgeLength(self, size=None, sizes=None, frames=None, identity=False, log=False):
        """ma::getMaximumEdgeLength(m, sf): identity=True is the reference's sf = 0
        (IdentitySizeField); otherwise the isotropic (size, None = resident) or
        anisotropic (sizes, frames; log=True: LogAnisoSizeField) field."""
        kind, s, ss, ff = self._size_kind(size, sizes, frames, identity, log)
        out = ctypes.c_double()
        self._check(self._lib.sprg_get_maximum_edge_length(self.h, kind, self._ptr(s), self._ptr(ss), self._ptr(ff),
                                                           ctypes.byref(out)))
        return out.value

    def getAverageEdgeLength(self):
        """ma::getAverageEdgeLength(m): mean apf::measure of the edges."""
        out = ctypes.c_double()
        self._check(self._lib.sprg_get_average_edge_length(self.h, ctypes.byref(out)))
        return out.value

    def markBadQuality(self, good_quality, flags):
        """ma::markBadQuality on the qualities of the last measureQuality; element
        flags (int32, n_elems) updated in place.  Returns the marked count."""
        if flags.dtype != np.int32 or not flags.flags["C_CONTIGUOUS"]:
            raise TypeError("flags must be a contiguous int32 array")
        n = ctypes.c_long()
        self._check(self._lib.sprg_mark_bad_quality(self.h, float(good_quality), flags.ctypes.data, ctypes.byref(n)))
        return n.value

    def getMinQuality(self):
        """ma::getMinQuality on the qualities of the last measureQuality."""
        out = ctypes.c_double()
        self._check(self._lib.sprg_get_min_quality(self.h, ctypes.byref(out)))
        return out.value

    def collapseSizeCheck(self, keep, edges, adjacent, size=None, sizes=None, frames=None):
        """ma::collapseSizeCheck (ma/maCoarsen.cc:47-60) for a batch of candidate
        collapses: collapse i keeps vertex keep[i] and removes the other vertex
        of edges[i]; adjacent[i] lists the edges the reference passes as
        `adjacent`.  The new edges run from the kept vertex to the vertex of each
        adjacent edge opposite the collapsing one; all are measured in one
        launch.  Returns one bool per collapse (no new edge longer than 1.5)."""
        ev = self.mesh.edge_verts
        pairs, owner = [], []
        for i, (k, e) in enumerate(zip(keep, edges)):
            a, b = int(ev[e][0]), int(ev[e][1])
            vc = b if a == k else a
            for f in adjacent[i]:
                p, q = int(ev[f][0]), int(ev[f][1])
                pairs.append((k, q if p == vc else p))
                owner.append(i)
        ok = np.ones(len(keep), bool)
        if pairs:
            L = self.measure_vertex_pairs(np.array(pairs, np.int32), size, sizes, frames)
            np.logical_and.at(ok, np.array(owner), ~(L > 1.5))
        return ok

    # -- the whole pass --------------------------------------------------
    def estimate_and_mark(self, u, adapt_ratio, flags=None, size_out=None):
        """getGradIPField -> getSPRSizeField -> makeSizeField -> collapse/split marks.
        Returns (size, flags, n_split, n_collapse, info); size_out (float64,
        n_verts, e.g. pinned) receives the size field when given."""
        u = _f64(u)
        if flags is None:
            flags = np.zeros(self.mesh.n_edges, np.int32)
        if size_out is not None and (size_out.dtype != np.float64 or size_out.shape != (self.mesh.n_verts,)
                                     or not size_out.flags["C_CONTIGUOUS"]):
            raise TypeError("size_out must be a contiguous float64 array of n_verts")
        size = np.empty(self.mesh.n_verts, np.float64) if size_out is None else size_out
        ns, nc = ctypes.c_long(), ctypes.c_long()
        info = _lib.SizeInfo()
        self._check(self._lib.sprg_estimate_and_mark(self.h, u.ctypes.data, float(adapt_ratio), size.ctypes.data,
                                                     flags.ctypes.data, ctypes.byref(ns), ctypes.byref(nc),
                                                     ctypes.byref(info)))
        return size, flags, ns.value, nc.value, info.as_dict()

    # ---- launch shape and graphs ---------------------------------------------
    def set_autotune(self, on=True):
        self._check(self._lib.sprg_set_autotune(self.h, 1 if on else 0))

    def set_tiling(self, lanes, tile_verts=256, blocks_per_sm=8):
        """Fix the binned recovery's shape: lanes per vertex for each of the
        four patch-size bins (1, 2, 4, or 0 for the sliced patch lists, which
        needs tile_verts a multiple of 32)."""
        l = np.ascontiguousarray(lanes, np.int32)
        self._check(self._lib.sprg_set_tiling(self.h, l.ctypes.data, int(tile_verts), int(blocks_per_sm)))

    def tuning_report(self):
        import json
        return json.loads(self._lib.sprg_tuning_report(self.h).decode())

    def graph_capture(self, d_u, adapt_ratio, d_split_bits, d_collapse_bits):
        """Capture the resident pass into a CUDA graph (needs set_stream)."""
        self._check(self._lib.sprg_graph_capture(self.h, d_u, float(adapt_ratio), d_split_bits, d_collapse_bits))

    def graph_replay(self):
        self._check(self._lib.sprg_graph_replay(self.h))

    # ---- batch of meshes ---------------------------------------------------
    def set_batch(self, vert_offsets, elem_offsets, adapt_ratios):
        """Treat the context's mesh as a disjoint union of meshes (prefix
        offsets of length n + 1) with per-mesh adapt ratios."""
        vo = np.ascontiguousarray(vert_offsets, np.int64)
        eo = np.ascontiguousarray(elem_offsets, np.int64)
        r = np.ascontiguousarray(adapt_ratios, np.float64)
        self._check(self._lib.sprg_set_batch(self.h, int(r.size), vo.ctypes.data, eo.ctypes.data, r.ctypes.data))
        self._batch_n = int(r.size)

    def batch_info(self):
        """(n, 3): eps_star_norm2, error_sum, size_factor per mesh."""
        out = np.empty((self._batch_n, 3))
        self._check(self._lib.sprg_batch_info(self.h, out.ctypes.data))
        return out

    def hessian_metric(self, hessian, eps, h_min, h_max):
        """(sizes V x 3, frames V x 9) from a nodal Hessian V x 9."""
        V = self.mesh.n_verts
        H = _f64(hessian, (V, 9))
        sizes = np.empty((V, 3))
        frames = np.empty((V, 9))
        self._check(self._lib.sprg_hessian_metric(self.h, H.ctypes.data, float(eps), float(h_min), float(h_max),
                                                  sizes.ctypes.data, frames.ctypes.data))
        return sizes, frames

    def aniso_estimate_and_mark_resident(self, d_u, eps, h_min, h_max, d_split_bits, d_collapse_bits, d_quality=None):
        """The anisotropic pass on device pointers (FP64)."""
        self._check(self._lib.sprg_aniso_estimate_and_mark_resident(
            self.h, d_u, float(eps), float(h_min), float(h_max), d_split_bits, d_collapse_bits, d_quality))

    def estimate_and_mark_resident(self, d_u, adapt_ratio, d_split_bits, d_collapse_bits):
        """Device-pointer form (ints are raw device addresses); asynchronous."""
        self._check(self._lib.sprg_estimate_and_mark_resident(self.h, ctypes.c_void_p(d_u), float(adapt_ratio),
                                                              ctypes.c_void_p(d_split_bits),
                                                              ctypes.c_void_p(d_collapse_bits)))

    def rounding_dominated(self):
        """After an FP32 resident pass on one mesh: True when the reference's
        own FP64 rounding would decide its sizes (rerun under FP64 for its
        marks)."""
        v = ctypes.c_int(0)
        self._check(self._lib.sprg_rounding_dominated(self.h, ctypes.byref(v)))
        return bool(v.value)


class SizeField:
    """ma::SizeField over a context (IsoUserField, AnisoSizeField or LogAnisoSizeField)."""

    def __init__(self, ctx, size=None, sizes=None, frames=None, log=False):
        self.ctx, self.size, self.sizes, self.frames, self.log = ctx, size, sizes, frames, log

    def measure(self):
        """MetricSizeField::measure of every edge (MDS edge order)."""
        if self.sizes is not None and self.log:
            return self.ctx.measure_edges_log_aniso(self.sizes, self.frames)
        if self.sizes is not None:
            return self.ctx.measure_edges_aniso(self.sizes, self.frames)
        return self.ctx.measure_edges(self.size)

    def shouldSplit(self):
        return self.measure() > 1.5

    def shouldCollapse(self):
        return self.measure() < 0.5


def mesh_delta(old, new):
    """Rows of `new`'s flattened arrays that differ from `old`'s or lie beyond
    its counts: {vert_ids, coords, elem_ids, elem_verts, edge_ids,
    edge_verts} (int32 ids, contiguous values)."""
    def rows(a_old, a_new, dtype):
        a_old = np.asarray(a_old)
        a_new = np.ascontiguousarray(a_new, dtype)
        n_old, n_new = a_old.shape[0], a_new.shape[0]
        k = min(n_old, n_new)
        changed = np.nonzero(np.any(a_old[:k].reshape(k, -1) != a_new[:k].reshape(k, -1), axis=1))[0]
        ids = np.concatenate([changed, np.arange(k, n_new)]).astype(np.int32)
        return ids, np.ascontiguousarray(a_new[ids])
    vi, vx = rows(old.coords, new.coords, np.float64)
    ei, ex = rows(old.elem_verts, new.elem_verts, np.int32)
    di, dx = rows(old.edge_verts, new.edge_verts, np.int32)
    return {"vert_ids": vi, "coords": vx, "elem_ids": ei, "elem_verts": ex, "edge_ids": di, "edge_verts": dx}


def max_iterations_for_length(max_metric_length):
    """The maximumIterations ma::configure derives from the maximum metric edge
    length (updateMaxIterBasedOnSize, ma/maInput.cc:174-190)."""
    return int(_lib.load().sprg_max_iterations_for_length(float(max_metric_length)))


def apply_marks(split_bits, collapse_bits, flags):
    """Host write-back of the device edge-mark bitmaps into ma_flags words."""
    lib = _lib.load()
    ns, nc = ctypes.c_long(), ctypes.c_long()
    sb = None if split_bits is None else np.ascontiguousarray(split_bits, np.uint32)
    cb = None if collapse_bits is None else np.ascontiguousarray(collapse_bits, np.uint32)
    check(lib.sprg_apply_marks(flags.shape[0], None if sb is None else sb.ctypes.data,
                               None if cb is None else cb.ctypes.data, flags.ctypes.data, ctypes.byref(ns),
                               ctypes.byref(nc)))
    return ns.value, nc.value

"""Host runtime over the C ABI: context, device pattern, SpMV.

torch is used only for device memory and streams.  Every compute call goes
through libsimit_gb300.so.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from ._lib import F32, F64, P, call

_TORCH_DT = {F32: torch.float32, F64: torch.float64}


def dtype_code(t):
    if t.dtype == torch.float64:
        return F64
    if t.dtype == torch.float32:
        return F32
    raise TypeError("unsupported dtype %s" % t.dtype)


def ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else ctypes.c_void_p(0)


class Context:
    """One sg_ctx: a device and its stream.  `torch_stream` lets torch ops be
    ordered on the same stream (use `with ctx.stream():`, or make it current).
    Tensors handed to the C ABI must be allocated and written on this stream
    (or synchronised with it): the C ABI's kernels run on it, and torch's
    caching allocator only orders reuse within one stream."""

    def __init__(self, device=0):
        _lib.load()
        torch.cuda.init()
        h = P()
        call("sg_ctx_create", device, ctypes.byref(h))
        self.h = h
        self.device = torch.device("cuda", device)
        self.torch_stream = torch.cuda.ExternalStream(_lib.load().sg_ctx_stream(h),
                                                      device=self.device)

    def stream(self):
        return torch.cuda.stream(self.torch_stream)

    def sync(self):
        call("sg_ctx_sync", self.h)

    def close(self):
        if self.h:
            _lib.load().sg_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Pattern:
    """Blocked-CSR pattern of `map f to E` plus incidence and slot map, built
    on the device (sg_incidence_build / sg_pattern_count / sg_pattern_fill /
    sg_slots_build)."""

    def __init__(self, ctx, n, endpoints, card, with_slots=True):
        dev = ctx.device
        with ctx.stream():
            ep = torch.as_tensor(np.ascontiguousarray(endpoints, np.int32)) \
                if not isinstance(endpoints, torch.Tensor) else endpoints
            ep = ep.to(device=dev, dtype=torch.int32).contiguous()
        nE = ep.numel() // card
        self.n, self.card, self.nE, self.endpoints = n, card, nE, ep
        with ctx.stream():
            self.ve_ptr = torch.empty(n + 1, dtype=torch.int32, device=dev)
            self.ve_idx = torch.empty(max(1, nE * card), dtype=torch.int32, device=dev)
            self.rowptr = torch.empty(n + 1, dtype=torch.int32, device=dev)
        call("sg_incidence_build", ctx.h, n, ptr(ep), nE, card, ptr(self.ve_ptr),
             ptr(self.ve_idx))
        nnzb = ctypes.c_int64()
        call("sg_pattern_count", ctx.h, n, ptr(ep), nE, card, ptr(self.ve_ptr),
             ptr(self.ve_idx), ptr(self.rowptr), ctypes.byref(nnzb))
        self.nnzb = nnzb.value
        with ctx.stream():
            self.colidx = torch.empty(max(1, self.nnzb), dtype=torch.int32, device=dev)
        call("sg_pattern_fill", ctx.h, n, ptr(ep), nE, card, ptr(self.ve_ptr),
             ptr(self.ve_idx), ptr(self.rowptr), ptr(self.colidx))
        self.slots = None
        if with_slots:
            with ctx.stream():
                self.slots = torch.empty(max(1, nE * card * card), dtype=torch.int32, device=dev)
            call("sg_slots_build", ctx.h, n, ptr(ep), nE, card, ptr(self.rowptr),
                 ptr(self.colidx), ptr(self.slots))

    def host(self):
        """(rowptr, colidx) as uint32 numpy arrays."""
        rp = self.rowptr.cpu().numpy().view(np.uint32)
        ci = self.colidx[:self.nnzb].cpu().numpy().view(np.uint32)
        return rp, ci


def bspmv(ctx, n, bs, rowptr, colidx, vals, x, y=None, g=0):
    """y [n*bs] = A x for n block rows (x is indexed by column, so its length
    is the column count times bs: a rectangular matrix's differs from n*bs)."""
    if y is None:
        with ctx.stream():
            y = torch.empty(n * bs, dtype=x.dtype, device=x.device)
    if y.numel() < n * bs or y.dtype != x.dtype:
        raise ValueError("bspmv: y needs %d %s entries" % (n * bs, x.dtype))
    call("sg_bspmv", ctx.h, n, bs, ptr(rowptr), ptr(colidx), dtype_code(vals), ptr(vals),
         dtype_code(x), ptr(x), ptr(y), g)
    return y


def bsr_add_diag(ctx, n, bs, rowptr, colidx, vals, diag=None, ident=0.0, scale=1.0, out=None):
    """System-matrix expression D + scale*K on K's pattern (`MDK = MD + K`):
    diag [n*bs*bs] Diagonal storage or, with diag None, ident*I.  out may be
    vals (in place).  Values and diag share vals' dtype."""
    if out is None:
        with ctx.stream():
            out = torch.empty_like(vals)
    if diag is not None:
        assert diag.dtype == vals.dtype and diag.numel() == n * bs * bs
    call("sg_bsr_add_diag", ctx.h, n, bs, ptr(rowptr), ptr(colidx), vals.numel() // (bs * bs),
         dtype_code(vals), ptr(diag), float(ident), float(scale), ptr(vals), ptr(out))
    return out


class SymBsr:
    """sg_symbsr: symmetric (upper-half) storage of a 3x3-blocked FP32 matrix
    with a symmetric pattern; fill() from full values, spmv() = A x."""

    def __init__(self, ctx, n, rowptr, colidx, nnzb, stages=0):
        self.ctx, self.n = ctx, n
        self._keep = (rowptr, colidx)
        h = ctypes.c_void_p()
        call("sg_symbsr_create", ctx.h, n, ptr(rowptr), ptr(colidx), int(nnzb), int(stages),
             ctypes.byref(h))
        self.h = h.value

    def fill(self, vals):
        assert vals.dtype == torch.float32
        self._vals = vals
        call("sg_symbsr_fill", self.h, ptr(vals))

    def spmv(self, x, y=None):
        if x.numel() != self.n * 3 or x.dtype != torch.float32:
            raise ValueError("symmetric spmv: x needs %d float32 entries" % (self.n * 3))
        if y is None:
            with self.ctx.stream():
                y = torch.empty(self.n * 3, dtype=torch.float32, device=x.device)
        if y.numel() < self.n * 3:
            raise ValueError("symmetric spmv: y needs %d entries" % (self.n * 3))
        call("sg_symbsr_spmv", self.h, ptr(x), ptr(y))
        return y

    def close(self):
        if self.h:
            _lib.load().sg_symbsr_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def residual(ctx, n, bs, rowptr, colidx, vals, nnzb, x, b, mode=_lib.RESIDUAL_FP64):
    """r = b - A x (FP64 x, b) and ||r||^2 through sg_residual."""
    A = _lib.Matrix(n, bs, nnzb, rowptr.data_ptr(), colidx.data_ptr(), dtype_code(vals),
                    vals.data_ptr())
    with ctx.stream():
        r = torch.empty_like(b)
    rr = ctypes.c_double()
    call("sg_residual", ctx.h, ctypes.byref(A), ptr(x), ptr(b), ptr(r), ctypes.byref(rr),
         int(mode))
    return r, rr.value


class IncidenceMatrix:
    """An edge set's incidence pattern over one vertex set (sg_incidence_pattern):
    kind INCIDENCE_EV (rows = elements, tensor[E,V]) or INCIDENCE_VE (rows =
    vertices, tensor[V,E]).  sel [nE*npos]: each element's endpoints in that
    vertex set, in endpoint order; n: the vertex set's size."""

    def __init__(self, ctx, kind, n, sel, npos):
        d = ctx.device
        self.ctx, self.kind, self.n, self.npos = ctx, kind, n, npos
        with ctx.stream():
            self.sel = torch.as_tensor(np.ascontiguousarray(sel, np.int32)).to(d)
        self.nE = self.sel.numel() // npos
        m = self.nE * npos
        self.rows = self.nE if kind == _lib.INCIDENCE_EV else n
        with ctx.stream():
            self.rowptr = torch.empty(self.rows + 1, dtype=torch.int32, device=d)
            self.colidx = torch.empty(max(1, m), dtype=torch.int32, device=d)
            self.slot_of = torch.empty(max(1, m), dtype=torch.int32, device=d)
        call("sg_incidence_pattern", ctx.h, kind, n, self.nE, npos, ptr(self.sel),
             ptr(self.rowptr), ptr(self.colidx), ptr(self.slot_of))
        self.nnzb = m

    def assemble(self, eb, bs, dtype=torch.float64):
        """Values [nnzb*bs*bs] from the element function's blocks eb [nE, npos, bs, bs]."""
        with self.ctx.stream():
            eb = _d(eb, dtype, self.ctx.device)
            vals = torch.empty(max(1, self.nnzb * bs * bs), dtype=dtype, device=self.ctx.device)
        call("sg_assemble_incidence", self.ctx.h, self.kind, self.nE, self.npos, ptr(self.sel),
             ptr(self.slot_of), dtype_code(vals), int(bs), ptr(eb), ptr(vals))
        return vals

    def spmv(self, bs, vals, x):
        cols = self.n if self.kind == _lib.INCIDENCE_EV else self.nE
        if x.numel() != cols * bs:
            raise ValueError("incidence spmv: x needs %d entries" % (cols * bs))
        return bspmv(self.ctx, self.rows, bs, self.rowptr, self.colidx, vals, x)


class RectMatrix:
    """matrix[Vr, Vc] of `map f to E` for an edge set over two vertex sets
    (sg_pattern_rect): sel_r [nE*npos_r] / sel_c [nE*npos_c] are each
    element's endpoints in the row and column sets; nr, nc their sizes."""

    def __init__(self, ctx, nr, nc, sel_r, npos_r, sel_c, npos_c):
        d = ctx.device
        self.ctx, self.nr, self.nc, self.npos_r, self.npos_c = ctx, nr, nc, npos_r, npos_c
        with ctx.stream():
            self.sel_r = torch.as_tensor(np.ascontiguousarray(sel_r, np.int32)).to(d)
            self.sel_c = torch.as_tensor(np.ascontiguousarray(sel_c, np.int32)).to(d)
        self.nE = self.sel_r.numel() // npos_r
        assert self.sel_c.numel() == self.nE * npos_c
        with ctx.stream():
            self.ve_ptr = torch.empty(nr + 1, dtype=torch.int32, device=d)
            self.ve_idx = torch.empty(max(1, self.nE * npos_r), dtype=torch.int32, device=d)
            self.rowptr = torch.empty(nr + 1, dtype=torch.int32, device=d)
        call("sg_incidence_build", ctx.h, nr, ptr(self.sel_r), self.nE, npos_r, ptr(self.ve_ptr),
             ptr(self.ve_idx))
        nnzb = ctypes.c_int64()
        args = (ctx.h, nr, nc, self.nE, npos_r, npos_c, ptr(self.sel_c), ptr(self.ve_ptr),
                ptr(self.ve_idx), ptr(self.rowptr))
        call("sg_pattern_rect", *args, None, ctypes.byref(nnzb))
        self.nnzb = nnzb.value
        with ctx.stream():
            self.colidx = torch.empty(max(1, self.nnzb), dtype=torch.int32, device=d)
        call("sg_pattern_rect", *args, ptr(self.colidx), ctypes.byref(nnzb))

    def assemble(self, eb, bs, dtype=torch.float64):
        """Values [nnzb*bs*bs] from blocks eb [nE, npos_r, npos_c, bs, bs]."""
        with self.ctx.stream():
            eb = _d(eb, dtype, self.ctx.device)
            vals = torch.empty(max(1, self.nnzb * bs * bs), dtype=dtype, device=self.ctx.device)
        call("sg_assemble_rect", self.ctx.h, self.nr, self.npos_r, self.npos_c, ptr(self.sel_c),
             ptr(self.ve_ptr), ptr(self.ve_idx), ptr(self.rowptr), ptr(self.colidx),
             dtype_code(vals), int(bs), ptr(eb), ptr(vals))
        return vals

    def spmv(self, bs, vals, x):
        if x.numel() != self.nc * bs:
            raise ValueError("rect spmv: x needs %d entries" % (self.nc * bs))
        return bspmv(self.ctx, self.nr, bs, self.rowptr, self.colidx, vals, x)


def check_element_source(element_src, card, bs, dtype=torch.float64, exact=True, vector=False):
    """Compiles an element function as JitAssembly (vector=False:
    element_block) or JitVectorAssembly (vector=True: element_vector) would
    (NVRTC, sm_103a) without a context or a GPU; returns the compiler log,
    raises SimitError with the log when the source does not compile."""
    buf = ctypes.create_string_buffer(8192)
    call("sg_jit_check_vector_source" if vector else "sg_jit_check_source",
         element_src.encode(), card, bs, F64 if dtype == torch.float64 else F32, int(exact),
         buf, len(buf))
    return buf.value.decode(errors="replace")


class JitAssembly:
    """`map f to E reduce +` with the element function given as CUDA source
    (sg_jit_assembly_create: compiled by NVRTC with a row-owner assembly
    kernel).  assemble(mesh, fields) -> values [nnzb*bs*bs]."""

    def __init__(self, ctx, element_src, card, bs, dtype=torch.float64, exact=True):
        self.ctx, self.card, self.bs, self.dtype = ctx, card, bs, dtype
        h = ctypes.c_void_p()
        call("sg_jit_assembly_create", ctx.h, element_src.encode(), card, bs,
             F64 if dtype == torch.float64 else F32, int(exact), ctypes.byref(h))
        self.h = h.value

    def assemble(self, mesh, fields, out=None):
        """fields: up to 8 arrays; floating-point ones are passed in the
        assembly's dtype, boolean ones as one byte per value, other integer
        ones (constraint flags) as int32.  `out` (nnzb*bs*bs values) is
        overwritten when given."""
        with self.ctx.stream():
            fields = [_d(f, self.dtype, self.ctx.device) if _is_float(f) else
                      _d(f, torch.bool if _is_bool(f) else torch.int32, self.ctx.device)
                      for f in fields]
            self._keep = fields
            arr = (ctypes.c_void_p * max(1, len(fields)))(*[f.data_ptr() for f in fields])
            vals = out if out is not None else mesh.empty(mesh.nnzb * self.bs * self.bs,
                                                          self.dtype)
            if vals.numel() < mesh.nnzb * self.bs * self.bs or vals.dtype != self.dtype:
                raise ValueError("jit assemble: out needs %d %s values" %
                                 (mesh.nnzb * self.bs * self.bs, self.dtype))
            call("sg_jit_assemble", self.h, mesh.ref(), arr, len(fields), ptr(vals))
            return vals

    def close(self):
        if self.h:
            _lib.load().sg_jit_assembly_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class JitVectorAssembly(JitAssembly):
    """`map f to E reduce +` into a system vector with the element function
    given as CUDA source (sg_jit_vector_create: element_vector, compiled by
    NVRTC with a vertex-owner kernel).  assemble(mesh, fields) -> values
    [n*bs]."""

    def __init__(self, ctx, element_src, card, bs, dtype=torch.float64, exact=True):
        self.ctx, self.card, self.bs, self.dtype = ctx, card, bs, dtype
        h = ctypes.c_void_p()
        call("sg_jit_vector_create", ctx.h, element_src.encode(), card, bs,
             F64 if dtype == torch.float64 else F32, int(exact), ctypes.byref(h))
        self.h = h.value

    def assemble(self, mesh, fields, out=None):
        with self.ctx.stream():
            fields = [_d(f, self.dtype, self.ctx.device) if _is_float(f) else
                      _d(f, torch.bool if _is_bool(f) else torch.int32, self.ctx.device)
                      for f in fields]
            self._keep = fields
            arr = (ctypes.c_void_p * max(1, len(fields)))(*[f.data_ptr() for f in fields])
            vals = out if out is not None else torch.empty(mesh.n * self.bs, dtype=self.dtype,
                                                           device=self.ctx.device)
            if vals.numel() < mesh.n * self.bs or vals.dtype != self.dtype:
                raise ValueError("jit assemble_vector: out needs %d %s values" %
                                 (mesh.n * self.bs, self.dtype))
            call("sg_jit_assemble_vector", self.h, mesh.ref(), arr, len(fields), ptr(vals))
            return vals


def _is_float(a):
    if isinstance(a, torch.Tensor):
        return a.is_floating_point()
    return np.asarray(a).dtype.kind == "f"


def _is_bool(a):
    if isinstance(a, torch.Tensor):
        return a.dtype == torch.bool
    return np.asarray(a).dtype.kind == "b"


def dot(ctx, a, b):
    out = ctypes.c_double()
    call("sg_dot", ctx.h, a.numel(), dtype_code(a), ptr(a), ptr(b), ctypes.byref(out))
    return out.value


def assemble_cloth_stretch(mesh, x, K, rest, dtype=torch.float64):
    """The cloth example's stretching force over a face mesh (card 3):
    f [n*3] (sg_assemble_cloth_stretch)."""
    d = mesh.ctx.device
    with mesh.ctx.stream():
        xs, Ks, rs = (_d(a, dtype, d) for a in (x, K, rest))
        f = torch.empty(mesh.n * 3, dtype=dtype, device=d)
    call("sg_assemble_cloth_stretch", mesh.ctx.h, mesh.ref(), dtype_code(f), ptr(xs), ptr(Ks),
         ptr(rs), ptr(f))
    return f


def assemble_cloth_bend(mesh, x, angle, length, perp, dtype=torch.float64):
    """The cloth example's bending force over a hinge mesh (card 4): f
    [n*3] (sg_assemble_cloth_bend)."""
    d = mesh.ctx.device
    with mesh.ctx.stream():
        xs, an, ln, pp = (_d(a, dtype, d) for a in (x, angle, length, perp))
        f = torch.empty(mesh.n * 3, dtype=dtype, device=d)
    call("sg_assemble_cloth_bend", mesh.ctx.h, mesh.ref(), dtype_code(f), ptr(xs), ptr(an),
         ptr(ln), ptr(pp), ptr(f))
    return f


def fp64_fma_rate(ctx):
    """sg_fp64_fma_rate: the device's FP64 FMA rate in TFLOP/s."""
    out = ctypes.c_double()
    call("sg_fp64_fma_rate", ctx.h, ctypes.byref(out))
    return out.value


def _host_f64(a):
    return (ctypes.c_double * len(a))(*[float(v) for v in a])


_ASM_TUNE_CACHE = {}


class Mesh:
    """A bound edge set + its device pattern, as the sg_mesh structure.

    plan: the element-parallel assembly plan that assembly with exact=False
    uses -- "gather" (element blocks written once, then every slot and
    vertex gathers its contributions in ascending element order), "colored"
    (blocks added into their slots colour by colour) -- or None (row-owner
    kernels).  colored=True is plan="colored"."""

    def __init__(self, ctx, n, endpoints, card, with_slots=False, colored=False, plan=None):
        self.ctx = ctx
        if colored and plan is None:
            plan = "colored"
        assert plan in (None, "colored", "gather"), plan
        self.pattern = Pattern(ctx, n, endpoints, card, with_slots=with_slots or plan is not None)
        p = self.pattern
        mr = ctypes.c_int32()
        call("sg_pattern_maxrow", ctx.h, n, ptr(p.rowptr), ctypes.byref(mr))
        self.maxrow = mr.value
        self.n, self.card, self.nE, self.nnzb = n, card, p.nE, p.nnzb
        self.s = _lib.Mesh(n, card, p.nE, p.endpoints.data_ptr(), p.ve_ptr.data_ptr(),
                           p.ve_idx.data_ptr(), p.rowptr.data_ptr(), p.colidx.data_ptr(),
                           p.nnzb, self.maxrow)
        self.ncolors = 0
        self.plan = plan
        if plan == "colored":
            self.color_plan()
        elif plan == "gather":
            self.gather_plan()

    def color_plan(self):
        """Slots + element colouring (sg_element_coloring) set in the sg_mesh."""
        p = self.pattern
        with self.ctx.stream():
            self.color_order = torch.empty(max(1, self.nE), dtype=torch.int32,
                                           device=self.ctx.device)
        self._color_ptr = (ctypes.c_int32 * (_lib.MAX_COLORS + 1))()
        nc = ctypes.c_int32()
        self.s.slots = p.slots.data_ptr()
        call("sg_element_coloring", self.ctx.h, ctypes.byref(self.s), ptr(self.color_order),
             ctypes.cast(self._color_ptr, ctypes.c_void_p), ctypes.byref(nc))
        self.ncolors = nc.value
        self.s.color_order = self.color_order.data_ptr()
        self.s.color_ptr = ctypes.cast(self._color_ptr, ctypes.c_void_p)
        self.s.ncolors = nc.value

    def gather_plan(self):
        """Slots + the inverse slot map (sg_slot_sources) set in the sg_mesh."""
        p = self.pattern
        self.s.slots = p.slots.data_ptr()
        with self.ctx.stream():
            self.slot_src_ptr = torch.empty(self.nnzb + 1, dtype=torch.int32,
                                            device=self.ctx.device)
            self.slot_src = torch.empty(max(1, self.nE * self.card * self.card),
                                        dtype=torch.int32, device=self.ctx.device)
        call("sg_slot_sources", self.ctx.h, ctypes.byref(self.s), ptr(self.slot_src_ptr),
             ptr(self.slot_src))
        self.s.slot_src_ptr = self.slot_src_ptr.data_ptr()
        self.s.slot_src = self.slot_src.data_ptr()

    def set_asm_tile(self, tile):
        """Element tile (threads per CTA) of the element-blocks plan."""
        assert tile in (0, 128, 256, 512)
        self.s.asm_tile = int(tile)

    def tune_assembly(self, assemble, plans=("gather", "colored", None), tiles=(128, 256, 512),
                      reps=3):
        """Assembly autotuner: times `assemble()` (the caller's assembly
        through this mesh) under every plan and, for the element-blocks plan,
        every element tile; keeps the fastest (plans are built as needed;
        the chosen one stays set).  The choice is cached per (n, nE, card,
        plan set).  Returns {"plan", "tile", "ms", "default_ms", "times"}."""
        key = (self.n, self.nE, self.card, tuple(plans), tuple(tiles))
        if key in _ASM_TUNE_CACHE:
            best = _ASM_TUNE_CACHE[key]
            self._use_plan(best["plan"])
            self.set_asm_tile(best["tile"])
            return dict(best, cached=True)
        times = {}
        st = self.ctx.torch_stream
        for plan in plans:
            self._use_plan(plan)
            for tile in (tiles if plan == "gather" else (0,)):
                self.set_asm_tile(tile)
                assemble()
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(st)
                for _ in range(reps):
                    assemble()
                e1.record(st)
                e1.synchronize()
                times["%s/%d" % (plan, tile)] = e0.elapsed_time(e1) / reps
        name = min(times, key=times.get)
        plan, tile = name.split("/")
        best = {"plan": None if plan == "None" else plan, "tile": int(tile), "ms": times[name],
                "default_ms": times.get("gather/256", times.get("gather/0")), "times": times}
        _ASM_TUNE_CACHE[key] = best
        self._use_plan(best["plan"])
        self.set_asm_tile(best["tile"])
        return dict(best, cached=False)

    def _use_plan(self, plan):
        """Switch the sg_mesh to a plan (building it once)."""
        p = self.pattern
        self.s.slots = self.s.color_order = self.s.color_ptr = None
        self.s.slot_src_ptr = self.s.slot_src = None
        self.s.ncolors = 0
        if plan == "colored":
            if getattr(self, "color_order", None) is None:
                self.color_plan()
            self.s.slots = p.slots.data_ptr()
            self.s.color_order = self.color_order.data_ptr()
            self.s.color_ptr = ctypes.cast(self._color_ptr, ctypes.c_void_p)
            self.s.ncolors = self.ncolors
        elif plan == "gather":
            if getattr(self, "slot_src", None) is None:
                self.gather_plan()
            self.s.slots = p.slots.data_ptr()
            self.s.slot_src_ptr = self.slot_src_ptr.data_ptr()
            self.s.slot_src = self.slot_src.data_ptr()
        self.plan = plan

    def colors(self):
        """(color_ptr list, color_order numpy) of the plan."""
        cp = [self._color_ptr[k] for k in range(self.ncolors + 1)]
        return cp, self.color_order[:self.nE].cpu().numpy()

    def ref(self):
        return ctypes.byref(self.s)

    def empty(self, count, dtype):
        with self.ctx.stream():
            return torch.zeros(max(1, count), dtype=dtype, device=self.ctx.device)


def _d(t, dtype, dev):
    if t is None:
        return None
    if isinstance(t, torch.Tensor):
        return t.to(device=dev, dtype=dtype).contiguous()
    return torch.as_tensor(np.ascontiguousarray(t)).to(device=dev, dtype=dtype).contiguous()


def assemble_springs(mesh, x, v, m, fixed, k, l0, h, viscous, grav, form=0,
                     dtype=torch.float64, exact=True):
    with mesh.ctx.stream():
        d = mesh.ctx.device
        x, v, m, k, l0 = (_d(a, dtype, d) for a in (x, v, m, k, l0))
        fixed = _d(fixed, torch.uint8, d)
        vals = mesh.empty(mesh.nnzb * 9, dtype)
        f = mesh.empty(mesh.n * 3, dtype)
        call("sg_assemble_springs", mesh.ctx.h, mesh.ref(), dtype_code(vals), form, ptr(x), ptr(v),
             ptr(m), ptr(fixed), ptr(k), ptr(l0), h, viscous, _host_f64(grav), ptr(vals), ptr(f),
             int(exact))
        return vals, f


def assemble_scalar_springs(mesh, a, diag, scale, dtype=torch.float64, exact=True):
    with mesh.ctx.stream():
        a = _d(a, dtype, mesh.ctx.device)
        vals = mesh.empty(mesh.nnzb, dtype)
        call("sg_assemble_scalar_springs", mesh.ctx.h, mesh.ref(), dtype_code(vals), ptr(a), diag,
             scale, ptr(vals), int(exact))
        return vals


def hilbert_order(coords, bits=10, curve="hilbert"):
    """vertex_ordering[old] = new (sg_hilbert_order, or sg_morton_order with
    curve="morton") of host coordinates [n*3]."""
    c = np.ascontiguousarray(coords, np.float64).reshape(-1)
    n = c.size // 3
    out = np.empty(n, np.int32)
    fn = {"hilbert": "sg_hilbert_order", "morton": "sg_morton_order"}[curve]
    call(fn, n, c.ctypes.data, int(bits), out.ctypes.data)
    return out


def element_order(endpoints, card):
    """element_order[new] = old (sg_element_order) of host endpoints."""
    ep = np.ascontiguousarray(endpoints, np.int32).reshape(-1)
    nE = ep.size // card
    out = np.empty(nE, np.int32)
    call("sg_element_order", nE, int(card), ep.ctypes.data, out.ctypes.data)
    return out


def reorder_mesh(n, endpoints, card, coords, bits=10, curve="hilbert"):
    """simit::reorder (src/reorder.cpp:252-273) of a host mesh: returns
    (vertex_ordering old->new, element_order new->old, new endpoints).
    Permute vertex fields with f_new[vo] = f_old and element fields with
    f_new = f_old[eo]."""
    vo = hilbert_order(coords, bits, curve)
    ep = vo[np.asarray(endpoints, np.int64).reshape(-1)].astype(np.int32)
    eo = element_order(ep, card)
    return vo, eo, ep.reshape(-1, card)[eo].reshape(-1)


def assemble_blocks(mesh, eb, bs, dtype=torch.float64, exact=True):
    """`map f to E reduce +` of caller-evaluated element blocks eb
    [nE, card, card, bs, bs] into the mesh's pattern (values [nnzb*bs*bs])."""
    with mesh.ctx.stream():
        eb = _d(eb, dtype, mesh.ctx.device).contiguous()
        vals = mesh.empty(mesh.nnzb * bs * bs, dtype)
        call("sg_assemble_blocks", mesh.ctx.h, mesh.ref(), dtype_code(vals), int(bs), ptr(eb),
             ptr(vals), int(exact))
        return vals


def tet_precompute(mesh, x, rho, dtype=torch.float64):
    with mesh.ctx.stream():
        x = _d(x, dtype, mesh.ctx.device)
        B = mesh.empty(mesh.nE * 9, dtype)
        W = mesh.empty(mesh.nE, dtype)
        m = mesh.empty(mesh.n, dtype)
        call("sg_tet_precompute", mesh.ctx.h, mesh.ref(), dtype_code(B), ptr(x), rho, ptr(B), ptr(W),
             ptr(m))
        return B, W, m


def assemble_tet_stiffness(mesh, model, x, c, B, W, mu, lam, h, rho, dtype=torch.float64,
                           exact=True):
    with mesh.ctx.stream():
        d = mesh.ctx.device
        x, B, W, mu, lam = (_d(a, dtype, d) for a in (x, B, W, mu, lam))
        c = _d(c, torch.int32, d)
        vals = mesh.empty(mesh.nnzb * 9, dtype)
        call("sg_assemble_tet_stiffness", mesh.ctx.h, mesh.ref(), dtype_code(vals), model, ptr(x),
             ptr(c), ptr(B), ptr(W), ptr(mu), ptr(lam), h, rho, ptr(vals), int(exact))
        return vals


def assemble_tet_force(mesh, model, x, v, c, B, W, mu, lam, h, rho, grav, dtype=torch.float64,
                       exact=True):
    with mesh.ctx.stream():
        d = mesh.ctx.device
        x, v, B, W, mu, lam = (_d(a, dtype, d) for a in (x, v, B, W, mu, lam))
        c = _d(c, torch.int32, d)
        f = mesh.empty(mesh.n * 3, dtype)
        call("sg_assemble_tet_force", mesh.ctx.h, mesh.ref(), dtype_code(f), model, ptr(x), ptr(v),
             ptr(c), ptr(B), ptr(W), ptr(mu), ptr(lam), h, rho, _host_f64(grav), ptr(f), int(exact))
        return f


def assemble_heat(mesh, B, W, kappa, dt, T0, dtype=torch.float64, exact=True):
    with mesh.ctx.stream():
        d = mesh.ctx.device
        B, W, kappa, T0 = (_d(a, dtype, d) for a in (B, W, kappa, T0))
        vals = mesh.empty(mesh.nnzb, dtype)
        b = mesh.empty(mesh.n, dtype)
        call("sg_assemble_heat", mesh.ctx.h, mesh.ref(), dtype_code(vals), ptr(B), ptr(W), ptr(kappa),
             dt, ptr(T0), ptr(vals), ptr(b), int(exact))
        return vals, b


def solve_opts(precision=_lib.SOLVE_F64, precond=_lib.PRECOND_NONE, stop=_lib.STOP_RELATIVE,
               tol=1e-8, maxiters=10000, verify=1, check_every=0, reliable_delta=0.1, lanes=0,
               batch=32, learned_params=None, learned_form=0, storage=0, pdl=0,
               learned_exec=_lib.MPNN_EXEC_FOLDED):
    lp = learned_params.data_ptr() if learned_params is not None else None
    return _lib.SolveOpts(precision, precond, stop, tol, maxiters, verify, check_every,
                          reliable_delta, lanes, batch, lp, int(learned_form), int(storage),
                          int(pdl), int(learned_exec))


class Solver:
    """sg_solver: set up once for a matrix, solve many right-hand sides."""

    def __init__(self, ctx, n, bs, rowptr, colidx, vals, nnzb, opts, learned_params_keep=None):
        self.ctx = ctx
        self._keep = (rowptr, colidx, vals)
        self.A = _lib.Matrix(n, bs, nnzb, rowptr.data_ptr(), colidx.data_ptr(),
                             dtype_code(vals), vals.data_ptr())
        self.opts = opts
        self._keep_params = learned_params_keep
        h = P()
        call("sg_solver_create", ctx.h, ctypes.byref(self.A), ctypes.byref(opts), ctypes.byref(h))
        self.h = h

    def solve(self, b, x):
        """b, x: FP64 device tensors (x = initial guess, overwritten)."""
        assert b.dtype == torch.float64 and x.dtype == torch.float64
        res = _lib.SolveResult()
        call("sg_solver_solve", self.h, ptr(b), ptr(x), ctypes.byref(res))
        return res

    def solve_ex(self, b, x, x_zero=False):
        """b FP32 or FP64 (widened by the solver), x FP64 (the guess unless
        x_zero; receives the solution)."""
        assert x.dtype == torch.float64 and b.dtype in (torch.float32, torch.float64)
        res = _lib.SolveResult()
        call("sg_solver_solve_ex", self.h, ptr(b), dtype_code(b), ptr(x), int(bool(x_zero)),
             ctypes.byref(res))
        return res

    def refresh(self):
        """The matrix values changed in place (re-assembly)."""
        call("sg_solver_refresh", self.h)

    def close(self):
        if self.h:
            _lib.load().sg_solver_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tune_spmv(ctx, n, bs, rowptr, colidx, vals, nnzb, xdt=torch.float32, reps=10, force=False):
    """sg_tune_spmv: {"g", "ms", "default_ms", "times": {g: ms}} of the
    fastest SpMV schedule on this matrix (cached per pattern unless force)."""
    A = _lib.Matrix(n, bs, nnzb, rowptr.data_ptr(), colidx.data_ptr(), dtype_code(vals),
                    vals.data_ptr())
    g = ctypes.c_int32()
    ms = ctypes.c_float()
    dms = ctypes.c_float()
    nc = ctypes.c_int32()
    cap = 64
    cg = (ctypes.c_int32 * cap)()
    cms = (ctypes.c_float * cap)()
    call("sg_tune_spmv", ctx.h, ctypes.byref(A), 1 if xdt == torch.float64 else 0, int(reps),
         int(bool(force)), ctypes.byref(g), ctypes.byref(ms), ctypes.byref(dms),
         ctypes.byref(nc), ctypes.cast(cg, ctypes.c_void_p), ctypes.cast(cms, ctypes.c_void_p),
         cap)
    times = {int(cg[k]): float(cms[k]) for k in range(min(nc.value, cap))}
    return {"g": g.value, "ms": ms.value, "default_ms": dms.value if nc.value else None,
            "times": times}

"""ctypes front end of the C oracle (``sem_oracle.c``).

TEST INFRASTRUCTURE ONLY: the checker the CUDA library is compared against,
and the timed CPU baseline.  Only the tests, the smoke check and the CPU
baseline leg of the benchmark use this module; the product never does.

Every function returns numpy arrays in Neko's field layout
``x(lx,ly,lz,nelv)`` flattened with i fastest (see ``sem_oracle.c``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle_sem.so")
_lib = None

_d = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_f = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_i32 = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_i64 = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")
_vp = C.c_void_p
_I64 = C.c_int64
_D = C.c_double


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    srcs = [os.path.join(_HERE, f) for f in ("sem_oracle.c", "terms_oracle.c", "mma_oracle.c", "Makefile")]
    if force or not os.path.exists(_LIB_PATH) or any(os.path.getmtime(_LIB_PATH) < os.path.getmtime(f) for f in srcs):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        L.orc_rng_u64.restype = C.c_uint64
        L.orc_rng_u64.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64]
        L.orc_rng_unif.restype = _D
        L.orc_rng_unif.argtypes = [C.c_uint64, C.c_uint64, C.c_uint64]
        L.orc_num_threads.restype = C.c_int
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_gll.argtypes = [C.c_int, _d, _d, _d]
        L.orc_deform_params.argtypes = [C.c_uint64, _vp, _d]
        L.orc_mesh_box.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _d, _d, _D, C.c_uint64, _d, _d, _d, _i64]
        L.orc_mask_face_xmax.restype = _I64
        L.orc_mask_face_xmax.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _vp]
        L.orc_geom.argtypes = [_I64, C.c_int, _d, _d, _d] + [_d] * 7 + [_vp]
        L.orc_gs_build.restype = _I64
        L.orc_gs_build.argtypes = [_I64, _i64, _i32, _i64, _vp]
        L.orc_gs_op.argtypes = [_d, _I64, _i32, _i64, C.c_int]
        L.orc_mult.argtypes = [_I64, _I64, _i32, _i64, _d]
        L.orc_ax_helm.argtypes = [_I64, C.c_int, _d, _d, _d] + [_d] * 6 + [_vp, _D, _vp, _d]
        L.orc_ax_helm_f32.argtypes = [_I64, C.c_int, _f, _f, _f] + [_f] * 6 + [_vp, C.c_float, _vp]
        L.orc_helm_diag.argtypes = [_I64, C.c_int, _d, _d] + [_d] * 6 + [_vp, _D, _vp, _d]
        L.orc_glsc3.restype = _D
        L.orc_glsc3.argtypes = [_I64, _d, _d, _d]
        L.orc_jacobi.argtypes = ([_I64, C.c_int, _d] + [_d] * 6 + [_vp, _D, _vp, _d] +
                                 [_I64, _i32, _i64, _vp, _I64, _d])
        cg_args = ([_I64, C.c_int, _d] + [_d] * 6 + [_vp, _D, _vp, _d, _d] +
                   [_I64, _i32, _i64, _vp, _I64, _d, _d, _d])
        L.orc_cg.argtypes = cg_args + [_D, _D, C.c_int, _d]
        L.orc_cg_time_per_iter.restype = _D
        L.orc_cg_time_per_iter.argtypes = cg_args + [C.c_int]
        L.orc_proj_pre.argtypes = [_I64, C.c_int, _vp, _vp, _d, _d, _d, _d]
        L.orc_proj_post.restype = C.c_int
        L.orc_proj_post.argtypes = [_I64, C.c_int, C.c_int, _d, _d, _d, _d, _d, _d, _d]
        L.orc_ramp_forward.argtypes = [_I64, _d, _d, _D, _D, _D, C.c_int]
        L.orc_ramp_backward.argtypes = [_I64, _d, _d, _d, _D, _D, _D, C.c_int]
        L.orc_brinkman.argtypes = [_I64, _d, _d, _d, _d, _d, _d, _d]
        L.orc_permeability.argtypes = [_I64, _d, _d, _D, _D, _D]
        L.orc_sens_min_dissipation.argtypes = [_I64, _d, _d, _d, _d, _d, _d, _d, C.c_int, _D]
        L.orc_cadd_mask.argtypes = [_d, _D, _i32, _I64]
        L.orc_invcol1_mask.argtypes = [_d, _i32, _I64]
        L.orc_cmult_mask.argtypes = [_d, _D, _i32, _I64]
        L.orc_col2_mask.argtypes = [_d, _d, _i32, _I64]
        L.orc_col3_mask.argtypes = [_d, _d, _d, _i32, _I64]
        L.orc_sub3_mask.argtypes = [_d, _d, _d, _i32, _I64]
        L.orc_glsc2_mask.restype = _D
        L.orc_glsc2_mask.argtypes = [_d, _d, _i32, _I64]
        L.orc_field_uniform.argtypes = [_I64, _i64, C.c_uint64, C.c_uint64, _D, _D, _d]
        L.orc_fourier_params.argtypes = [C.c_uint64, C.c_int, C.c_int, _vp, _d, _d]
        L.orc_field_fourier.argtypes = [_I64, _d, _d, _d, _d, _d, C.c_int, _vp, _d, _d, _d]
        L.orc_field_blobs.argtypes = [_I64, _d, _d, _d, _d, _d, C.c_uint64, C.c_int, _D, _d]
        _lib = L
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


STREAM_RHO, STREAM_RHS = 2, 3


def set_threads(t: int) -> None:
    lib().orc_set_threads(int(t))


def num_threads() -> int:
    return int(lib().orc_num_threads())


def gll(lx: int):
    xi = np.zeros(lx); w = np.zeros(lx); D = np.zeros(lx * lx)
    lib().orc_gll(lx, xi, w, D)
    return xi, w, D.reshape(lx, lx)


def mesh_box(ex, ey, ez, lx, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), amp=0.0, seed=0):
    n = ex * ey * ez * lx ** 3
    x = np.zeros(n); y = np.zeros(n); z = np.zeros(n); gid = np.zeros(n, dtype=np.int64)
    lib().orc_mesh_box(ex, ey, ez, lx, np.asarray(lo, dtype=np.float64), np.asarray(hi, dtype=np.float64),
                       float(amp), int(seed), x, y, z, gid)
    return x, y, z, gid


def mask_face_xmax(ex, ey, ez, lx):
    cnt = lib().orc_mask_face_xmax(ex, ey, ez, lx, None)
    m = np.zeros(cnt, dtype=np.int32)
    lib().orc_mask_face_xmax(ex, ey, ez, lx, _ptr(m))
    return m


@dataclass
class Mesh:
    """Everything the operator needs, built by the oracle."""
    ex: int
    ey: int
    ez: int
    lx: int
    lo: tuple
    hi: tuple
    amp: float
    seed: int
    x: np.ndarray = field(repr=False, default=None)
    y: np.ndarray = field(repr=False, default=None)
    z: np.ndarray = field(repr=False, default=None)
    gid: np.ndarray = field(repr=False, default=None)
    D: np.ndarray = field(repr=False, default=None)
    w: np.ndarray = field(repr=False, default=None)
    G: dict = field(repr=False, default=None)
    B: np.ndarray = field(repr=False, default=None)
    jac: np.ndarray = field(repr=False, default=None)
    perm: np.ndarray = field(repr=False, default=None)
    offs: np.ndarray = field(repr=False, default=None)
    uid: np.ndarray = field(repr=False, default=None)
    nu: int = 0
    mult: np.ndarray = field(repr=False, default=None)

    @property
    def nelv(self):
        return self.ex * self.ey * self.ez

    @property
    def n(self):
        return self.nelv * self.lx ** 3


def build_mesh(ex, ey, ez, lx=8, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), amp=0.0, seed=0) -> Mesh:
    m = Mesh(ex, ey, ez, lx, tuple(lo), tuple(hi), amp, seed)
    m.x, m.y, m.z, m.gid = mesh_box(ex, ey, ez, lx, lo, hi, amp, seed)
    xi, m.w, m.D = gll(lx)
    n = m.n
    G = {k: np.zeros(n) for k in ("g11", "g12", "g13", "g22", "g23", "g33")}
    m.B = np.zeros(n); m.jac = np.zeros(n)
    lib().orc_geom(m.nelv, lx, m.x, m.y, m.z, G["g11"], G["g12"], G["g13"], G["g22"], G["g23"], G["g33"],
                   m.B, _ptr(m.jac))
    m.G = G
    m.perm = np.zeros(n, dtype=np.int32)
    offs = np.zeros(n + 1, dtype=np.int64)
    m.uid = np.zeros(n, dtype=np.int32)
    m.nu = int(lib().orc_gs_build(n, m.gid, m.perm, offs, _ptr(m.uid)))
    m.offs = offs[: m.nu + 1].copy()
    m.mult = np.zeros(n)
    lib().orc_mult(n, m.nu, m.perm, m.offs, m.mult)
    return m


def mesh_slice(m: Mesh, e0: int, e1: int) -> Mesh:
    """The oracle Mesh of elements [e0, e1) of `m` (coordinates and global
    ids sliced, geometry and rank-local gather-scatter maps rebuilt): one
    rank's part of an element partition.  ex/ey/ez keep the box's x and y
    counts with ez = the slab's planes, so nelv = e1 - e0 for z-slabs."""
    return mesh_subset(m, np.arange(e0, e1), (m.ex, m.ey, (e1 - e0) // (m.ex * m.ey)))


def mesh_subset(m: Mesh, elems, dims=None) -> Mesh:
    """The oracle Mesh of the elements `elems` of `m` (any subset, in the
    given order): one rank's part of a general element partition.  `dims`
    (ex, ey, ez) with ex ey ez = len(elems) labels it; default (len, 1, 1)."""
    lx = m.lx
    nl = lx ** 3
    elems = np.asarray(elems, dtype=np.int64)
    ex, ey, ez = dims if dims is not None else (len(elems), 1, 1)
    s = Mesh(ex, ey, ez, lx, m.lo, m.hi, m.amp, m.seed)
    sel = (elems[:, None] * nl + np.arange(nl)[None, :]).ravel()
    s.x, s.y, s.z = (np.ascontiguousarray(a[sel]) for a in (m.x, m.y, m.z))
    s.gid = np.ascontiguousarray(m.gid[sel])
    s.w, s.D = m.w, m.D
    n = s.n
    G = {k: np.zeros(n) for k in ("g11", "g12", "g13", "g22", "g23", "g33")}
    s.B = np.zeros(n); s.jac = np.zeros(n)
    lib().orc_geom(s.nelv, lx, s.x, s.y, s.z, G["g11"], G["g12"], G["g13"], G["g22"], G["g23"], G["g33"],
                   s.B, _ptr(s.jac))
    s.G = G
    s.perm = np.zeros(n, dtype=np.int32)
    offs = np.zeros(n + 1, dtype=np.int64)
    s.uid = np.zeros(n, dtype=np.int32)
    s.nu = int(lib().orc_gs_build(n, s.gid, s.perm, offs, _ptr(s.uid)))
    s.offs = offs[: s.nu + 1].copy()
    s.mult = np.zeros(n)
    lib().orc_mult(n, s.nu, s.perm, s.offs, s.mult)
    return s


def mesh_general(x, y, z, gid, lx) -> Mesh:
    """The oracle Mesh of any hexahedral mesh given by its GLL node
    coordinates and global node ids (nelv x lx^3 each, x fastest)."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    nelv = x.size // lx ** 3
    s = Mesh(nelv, 1, 1, lx, (0.0, 0.0, 0.0), (1.0, 1.0, 1.0), 0.0, 0)
    s.x, s.y, s.z = x, np.ascontiguousarray(y, dtype=np.float64), np.ascontiguousarray(z, dtype=np.float64)
    s.gid = np.ascontiguousarray(gid, dtype=np.int64)
    _, s.w, s.D = gll(lx)
    n = s.n
    G = {k: np.zeros(n) for k in ("g11", "g12", "g13", "g22", "g23", "g33")}
    s.B = np.zeros(n); s.jac = np.zeros(n)
    lib().orc_geom(s.nelv, lx, s.x, s.y, s.z, G["g11"], G["g12"], G["g13"], G["g22"], G["g23"], G["g33"],
                   s.B, _ptr(s.jac))
    s.G = G
    s.perm = np.zeros(n, dtype=np.int32)
    offs = np.zeros(n + 1, dtype=np.int64)
    s.uid = np.zeros(n, dtype=np.int32)
    s.nu = int(lib().orc_gs_build(n, s.gid, s.perm, offs, _ptr(s.uid)))
    s.offs = offs[: s.nu + 1].copy()
    s.mult = np.zeros(n)
    lib().orc_mult(n, s.nu, s.perm, s.offs, s.mult)
    return s


def gs_op(m: Mesh, u: np.ndarray, op: int = 1) -> np.ndarray:
    v = np.ascontiguousarray(u, dtype=np.float64).copy()
    lib().orc_gs_op(v, m.nu, m.perm, m.offs, int(op))
    return v


def ax_helm(m: Mesh, u, h1=None, h1c=1.0, h2=None):
    w = np.zeros(m.n)
    G = m.G
    lib().orc_ax_helm(m.nelv, m.lx, m.D.ravel().copy(), w, np.ascontiguousarray(u, dtype=np.float64),
                      G["g11"], G["g12"], G["g13"], G["g22"], G["g23"], G["g33"],
                      _ptr(h1), float(h1c), _ptr(h2), m.B)
    return w


def ax_helm_f32(m: Mesh, u, h1=None, h1c=1.0, hB=None):
    f32 = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float32)
    w = np.zeros(m.n, dtype=np.float32)
    G = {k: f32(v) for k, v in m.G.items()}
    h1_, hB_ = f32(h1), f32(hB)
    lib().orc_ax_helm_f32(m.nelv, m.lx, f32(m.D.ravel()), w, f32(u),
                          G["g11"], G["g12"], G["g13"], G["g22"], G["g23"], G["g33"],
                          _ptr(h1_), float(h1c), _ptr(hB_))
    return w


def helm_diag(m: Mesh, h1=None, h1c=1.0, h2=None):
    d = np.zeros(m.n)
    G = m.G
    lib().orc_helm_diag(m.nelv, m.lx, m.D.ravel().copy(), d, G["g11"], G["g12"], G["g13"], G["g22"], G["g23"],
                        G["g33"], _ptr(h1), float(h1c), _ptr(h2), m.B)
    return d


def jacobi(m: Mesh, h1=None, h1c=1.0, h2=None, mask=None):
    dinv = np.zeros(m.n)
    G = m.G
    nm = 0 if mask is None else len(mask)
    lib().orc_jacobi(m.nelv, m.lx, m.D.ravel().copy(), G["g11"], G["g12"], G["g13"], G["g22"], G["g23"], G["g33"],
                     _ptr(h1), float(h1c), _ptr(h2), m.B, m.nu, m.perm, m.offs, _ptr(mask), nm, dinv)
    return dinv


def glsc3(a, b, c) -> float:
    return float(lib().orc_glsc3(len(a), np.ascontiguousarray(a, dtype=np.float64),
                                 np.ascontiguousarray(b, dtype=np.float64), np.ascontiguousarray(c, dtype=np.float64)))


def apply_mask_zero(v, mask):
    if mask is not None and len(mask):
        v[mask - 1] = 0.0
    return v


def assemble_rhs(m: Mesh, f_local, mask=None, weak=True):
    """b = mask(gs(B*f)) when weak, else mask(f) (f already assembled)."""
    b = np.ascontiguousarray(f_local * m.B if weak else f_local, dtype=np.float64)
    if weak:
        b = gs_op(m, b, 1)
    return apply_mask_zero(b, mask)


def cg(m: Mesh, f, x0=None, h1=None, h1c=1.0, h2=None, mask=None, dinv=None, rtol=1e-10, abstol=0.0,
       max_iter=800, fixed_iters=None):
    """Jacobi-PCG.  Returns (x, iterations, res_start, res_final)."""
    if dinv is None:
        dinv = jacobi(m, h1, h1c, h2, mask)
    x = np.zeros(m.n) if x0 is None else np.ascontiguousarray(x0, dtype=np.float64).copy()
    out = np.zeros(3)
    G = m.G
    nm = 0 if mask is None else len(mask)
    mi = -int(fixed_iters) if fixed_iters is not None else int(max_iter)
    lib().orc_cg(m.nelv, m.lx, m.D.ravel().copy(), G["g11"], G["g12"], G["g13"], G["g22"], G["g23"], G["g33"],
                 _ptr(h1), float(h1c), _ptr(h2), m.B, m.mult, m.nu, m.perm, m.offs, _ptr(mask), nm, dinv,
                 x, np.ascontiguousarray(f, dtype=np.float64), float(rtol), float(abstol), mi, out)
    return x, int(out[0]), float(out[1]), float(out[2])


def cg_time_per_iter(m: Mesh, f, iters, h1=None, h1c=1.0, h2=None, mask=None, dinv=None):
    if dinv is None:
        dinv = jacobi(m, h1, h1c, h2, mask)
    x = np.zeros(m.n)
    G = m.G
    nm = 0 if mask is None else len(mask)
    return float(lib().orc_cg_time_per_iter(
        m.nelv, m.lx, m.D.ravel().copy(), G["g11"], G["g12"], G["g13"], G["g22"], G["g23"], G["g33"],
        _ptr(h1), float(h1c), _ptr(h2), m.B, m.mult, m.nu, m.perm, m.offs, _ptr(mask), nm, dinv,
        x, np.ascontiguousarray(f, dtype=np.float64), int(iters)))


def op_apply(m: Mesh, u, h1=None, h1c=1.0, h2=None, mask=None):
    """Assembled, masked operator mask(gs(A u))."""
    return apply_mask_zero(gs_op(m, ax_helm(m, u, h1, h1c, h2)), mask)


class Projection:
    """Fischer residual projection (oracle side), basis size L."""

    def __init__(self, n, L):
        self.n, self.L, self.m = n, L, 0
        self.xs = np.zeros((L, n)); self.axs = np.zeros((L, n))

    def pre(self, b, mult):
        xbar = np.zeros(self.n); alpha = np.zeros(max(self.m, 1))
        b0 = b.copy()
        lib().orc_proj_pre(self.n, self.m, _ptr(self.xs), _ptr(self.axs), mult, b, xbar, alpha)
        self.xbar, self.axbar = xbar, b0 - b
        return b

    def post(self, dx, adx, mult):
        dx = np.ascontiguousarray(dx, dtype=np.float64).copy()
        self.m = int(lib().orc_proj_post(self.n, self.L, self.m, self.xs.ravel() if False else self._xs_flat(),
                                         self._axs_flat(), mult, dx, np.ascontiguousarray(adx, dtype=np.float64),
                                         self.xbar, self.axbar))
        return dx

    def _xs_flat(self):
        return self.xs.reshape(-1)

    def _axs_flat(self):
        return self.axs.reshape(-1)


def ramp_forward(xin, fmin, fmax, q, convex_up):
    out = np.zeros_like(xin)
    lib().orc_ramp_forward(len(xin), xin, out, fmin, fmax, q, int(convex_up))
    return out


def ramp_backward(xin, dF_dout, fmin, fmax, q, convex_up):
    out = np.zeros_like(xin)
    lib().orc_ramp_backward(len(xin), xin, dF_dout, out, fmin, fmax, q, int(convex_up))
    return out


def brinkman(fx, fy, fz, u, v, w, chi):
    fx, fy, fz = fx.copy(), fy.copy(), fz.copy()
    lib().orc_brinkman(len(fx), fx, fy, fz, u, v, w, chi)
    return fx, fy, fz


def permeability(phi, perm0, perm1, pen):
    out = np.zeros_like(phi)
    lib().orc_permeability(len(phi), phi, out, perm0, perm1, pen)
    return out


def sens_min_dissipation(u, v, w, ua, va, wa, if_lube=False, K_scale=0.0):
    s = np.zeros_like(u)
    lib().orc_sens_min_dissipation(len(u), s, u, v, w, ua, va, wa, int(if_lube), float(K_scale))
    return s


def masked(op, a, *args):
    """Apply one of the math_ext masked ops to a copy of a."""
    a = a.copy()
    getattr(lib(), "orc_" + op)(a, *args)
    return a


def glsc2_mask(a, b, mask):
    return float(lib().orc_glsc2_mask(a, b, mask, len(mask)))


def field_uniform(m: Mesh, seed, stream, lo, hi):
    f = np.zeros(m.n)
    lib().orc_field_uniform(m.n, m.gid, int(seed), int(stream), float(lo), float(hi), f)
    return f


def fourier_params(seed, nmodes, kmax=4):
    k = np.zeros(3 * nmodes, dtype=np.int32); amp = np.zeros(nmodes); ph = np.zeros(nmodes)
    lib().orc_fourier_params(int(seed), nmodes, kmax, _ptr(k), amp, ph)
    return k, amp, ph


def field_fourier(m: Mesh, k, amp, ph):
    f = np.zeros(m.n)
    k = np.ascontiguousarray(k, dtype=np.int32)
    lib().orc_field_fourier(m.n, m.x, m.y, m.z, np.asarray(m.lo, dtype=np.float64), np.asarray(m.hi, dtype=np.float64),
                            len(amp), _ptr(k), np.ascontiguousarray(amp), np.ascontiguousarray(ph), f)
    return f


def field_blobs(m: Mesh, seed, nblobs=12, width=0.1):
    f = np.zeros(m.n)
    lib().orc_field_blobs(m.n, m.x, m.y, m.z, np.asarray(m.lo, dtype=np.float64), np.asarray(m.hi, dtype=np.float64),
                          int(seed), int(nblobs), float(width), f)
    return f

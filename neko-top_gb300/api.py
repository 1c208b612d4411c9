"""Neko-shaped host interface over the C ABI.

Argument meaning, order and error behaviour follow the reference's call
sites (file:line given per class).  Device memory comes from torch CUDA
tensors; the library sees raw pointers only.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import torch

from ._native import (GS_OP_ADD, KSP_CG, KSP_CG_MIXED, KSP_FCG_MIXED, KSP_GMRES, KSP_GMRES_MIXED, NtgError, check,
                      check_last, lib, ntg_monitor)

_DT = {torch.float64: "f64", torch.float32: "f32", torch.int32: "i32", torch.int64: "i64"}


def _ptr(t, dtype=torch.float64, n=None, name="array"):
    if t is None:
        return None
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name}: expected a CUDA tensor")
    if t.dtype != dtype:
        raise TypeError(f"{name}: expected {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name}: must be contiguous")
    if n is not None and t.numel() != n:
        raise ValueError(f"{name}: expected {n} entries, got {t.numel()}")
    return C.c_void_p(t.data_ptr())


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


@dataclass
class ksp_monitor_t:
    """Neko's ksp_monitor_t (iter, res_start, res_final;
    sources/mapping_functions/PDE_filter_mapping.f90:265-272) plus the
    status and the mixed solver's inner/FP64 counts."""
    iter: int
    res_start: float
    res_final: float
    rhs_norm: float
    status: int
    inner_iter: int = 0
    fp64_ax: int = 0
    guess_rejected: int = 0

    @classmethod
    def from_c(cls, m: ntg_monitor):
        return cls(m.iter, m.res_start, m.res_final, m.rhs_norm, m.status, m.inner_iter, m.fp64_ax,
                   m.guess_rejected)


def mask_face_xmax(ex, ey, ez, lx, device="cuda"):
    """1-based local indices of the x = max face (a Dirichlet mask)."""
    n = C.c_int64(0)
    check(lib().ntg_mask_face_xmax(ex, ey, ez, lx, None, C.byref(n), None))
    m = torch.empty(n.value, dtype=torch.int32, device=device)
    check(lib().ntg_mask_face_xmax(ex, ey, ez, lx, _ptr(m, torch.int32), C.byref(n), _stream()))
    return m


def build_box(ex, ey, ez, lx=8, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), amp=0.0, seed=0, device="cuda"):
    """Synthetic box mesh (coordinates and global ids) on the device."""
    n = ex * ey * ez * lx ** 3
    x = torch.empty(n, dtype=torch.float64, device=device)
    y = torch.empty_like(x)
    z = torch.empty_like(x)
    gid = torch.empty(n, dtype=torch.int64, device=device)
    lo3 = (C.c_double * 3)(*lo)
    hi3 = (C.c_double * 3)(*hi)
    check(lib().ntg_mesh_box(ex, ey, ez, lx, lo3, hi3, float(amp), int(seed), _ptr(x), _ptr(y), _ptr(z),
                             _ptr(gid, torch.int64), _stream()))
    return x, y, z, gid


class coef_t:
    """Mesh + geometric factors + gather-scatter plan (Neko's coef_t and
    gs_t, built at sources/adjoint/adjoint_scheme.f90:341-343)."""

    def __init__(self, nelv, lx, x, y, z, glb_ids):
        n = nelv * lx ** 3
        h = C.c_void_p()
        check(lib().ntg_plan_create(C.byref(h), int(nelv), int(lx), _ptr(x, n=n, name="x"), _ptr(y, n=n, name="y"),
                                    _ptr(z, n=n, name="z"), _ptr(glb_ids, torch.int64, n, "glb_ids")))
        self._h = h
        check(lib().ntg_plan_set_stream(h, _stream()))
        ne, l, nn, nu, nsh = C.c_int64(), C.c_int(), C.c_int64(), C.c_int64(), C.c_int64()
        check(lib().ntg_plan_info(h, C.byref(ne), C.byref(l), C.byref(nn), C.byref(nu), C.byref(nsh)))
        self.nelv, self.lx, self.n, self.nu, self.nshared = ne.value, l.value, nn.value, nu.value, nsh.value
        self.device = x.device
        self.mask = None
        self.x, self.y, self.z, self.gid = x, y, z, glb_ids
        self._xyz = (x, y, z)  # for the derivative metrics, derived on first use
        self._metrics = False

    @classmethod
    def from_vertices(cls, ev, lx, x, y, z):
        """A plan for a general hexahedral mesh: ev (E x 8 numpy, global
        vertex ids in tensor corner order) numbers the GLL nodes
        (dofmap.dofmap_from_vertices); x, y, z are the node coordinates
        (CUDA tensors, Neko layout)."""
        import numpy as np
        from .dofmap import dofmap_from_vertices
        ev = np.asarray(ev)
        gid = torch.from_numpy(dofmap_from_vertices(ev, lx)).to(x.device)
        c = cls(ev.shape[0], lx, x, y, z, gid)
        c.x, c.y, c.z, c.gid = x, y, z, gid
        return c

    @classmethod
    def box(cls, ex, ey, ez, lx=8, lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), amp=0.0, seed=0, device="cuda"):
        x, y, z, gid = build_box(ex, ey, ez, lx, lo, hi, amp, seed, device)
        c = cls(ex * ey * ez, lx, x, y, z, gid)
        c.x, c.y, c.z, c.gid = x, y, z, gid
        c.box_dims = (ex, ey, ez)
        c.lo, c.hi = tuple(lo), tuple(hi)
        return c

    @property
    def handle(self):
        if self._h is None:
            raise NtgError(1, "coef_t used after free()")
        return self._h

    def set_coefs(self, h1=None, h1c=1.0, h2=None, h2c=0.0, ifh2=False):
        """coef%h1, coef%h2, coef%ifh2 (sources/mapping_functions/PDE_filter_mapping.f90:225-241)."""
        check(lib().ntg_coef_set(self.handle, _ptr(h1, n=self.n, name="h1"), float(h1c), _ptr(h2, n=self.n, name="h2"),
                                 float(h2c), int(bool(ifh2))))

    def set_mask(self, mask, base=1):
        """Dirichlet index list (bc_list); Neko masks are 1-based."""
        if mask is None or mask.numel() == 0:
            check(lib().ntg_plan_set_mask(self.handle, None, 0, int(base)))
            self.mask = None
            return
        check(lib().ntg_plan_set_mask(self.handle, _ptr(mask, torch.int32, name="mask"), mask.numel(), int(base)))
        self.mask = mask

    def metrics(self):
        """The cofactors drdx..dtdz, 1/jac and 1/gs(B) for the derivative
        operators (Neko's coef_t generate_dxyz / Binv), derived once."""
        if not self._metrics:
            x, y, z = self._xyz
            check(lib().ntg_metrics_set(self.handle, _ptr(x, n=self.n, name="x"), _ptr(y, n=self.n, name="y"),
                                        _ptr(z, n=self.n, name="z")))
            self._metrics = True
        return self

    def geometry(self):
        out = {k: torch.empty(self.n, dtype=torch.float64, device=self.device)
               for k in ("g11", "g12", "g13", "g22", "g23", "g33", "B", "mult")}
        check(lib().ntg_coef_get(self.handle, *[_ptr(out[k]) for k in ("g11", "g12", "g13", "g22", "g23", "g33", "B",
                                                                         "mult")]))
        torch.cuda.synchronize()
        return out

    # seeded synthetic fields on this mesh (the box keeps x, y, z, gid)
    def field_uniform(self, seed, stream_id, lo, hi):
        f = torch.empty(self.n, dtype=torch.float64, device=self.device)
        check(lib().ntg_field_uniform(_ptr(self.gid, torch.int64), self.n, int(seed), int(stream_id), float(lo),
                                      float(hi), _ptr(f), _stream()))
        return f

    def field_fourier(self, nmodes, seed, kmax=4):
        f = torch.empty(self.n, dtype=torch.float64, device=self.device)
        lo3, hi3 = (C.c_double * 3)(*self.lo), (C.c_double * 3)(*self.hi)
        check(lib().ntg_field_fourier(_ptr(self.x), _ptr(self.y), _ptr(self.z), self.n, lo3, hi3, int(nmodes),
                                      int(kmax), int(seed), _ptr(f), _stream()))
        return f

    def field_blobs(self, seed, nblobs=12, width=0.1):
        f = torch.empty(self.n, dtype=torch.float64, device=self.device)
        lo3, hi3 = (C.c_double * 3)(*self.lo), (C.c_double * 3)(*self.hi)
        check(lib().ntg_field_blobs(_ptr(self.x), _ptr(self.y), _ptr(self.z), self.n, lo3, hi3, int(seed),
                                    int(nblobs), float(width), _ptr(f), _stream()))
        return f

    def field_modes(self, k, amp, ph):
        """Fourier modes with explicit parameters (k: 3*m ints, amp, ph)."""
        import numpy as np
        k = np.ascontiguousarray(k, dtype=np.int32).ravel()
        amp = np.ascontiguousarray(amp, dtype=np.float64)
        ph = np.ascontiguousarray(ph, dtype=np.float64)
        f = torch.empty(self.n, dtype=torch.float64, device=self.device)
        lo3, hi3 = (C.c_double * 3)(*self.lo), (C.c_double * 3)(*self.hi)
        check(lib().ntg_field_modes(_ptr(self.x), _ptr(self.y), _ptr(self.z), self.n, lo3, hi3, len(amp),
                                    k.ctypes.data_as(C.POINTER(C.c_int)), amp.ctypes.data_as(C.POINTER(C.c_double)),
                                    ph.ctypes.data_as(C.POINTER(C.c_double)), _ptr(f), _stream()))
        return f

    def rhs_assemble(self, f):
        """b = mask(gs(B f)): the weak right-hand side of a source f."""
        b = torch.empty_like(f)
        check(lib().ntg_rhs_assemble(self.handle, _ptr(f, n=self.n), _ptr(b, n=self.n)))
        return b

    def gs_maps(self):
        perm = torch.empty(self.n, dtype=torch.int32, device=self.device)
        offs = torch.empty(self.nu + 1, dtype=torch.int64, device=self.device)
        check(lib().ntg_gs_export(self.handle, _ptr(perm, torch.int32), _ptr(offs, torch.int64)))
        torch.cuda.synchronize()
        return perm, offs

    def set_ax_path(self, use_tma: bool):
        """FP32 Ax: bulk-copy pipelined kernel (lx = 8) or the generic one."""
        check(lib().ntg_plan_set_ax_path(self.handle, int(bool(use_tma))))

    def set_gs_path(self, by_class: bool):
        """gather-scatter: multiplicity classes (default) or one thread per group."""
        check(lib().ntg_plan_set_gs_path(self.handle, int(bool(by_class))))

    def check_error(self) -> bool:
        f = C.c_int()
        check(lib().ntg_plan_check_error(self.handle, C.byref(f)))
        return bool(f.value)

    def free(self):
        if self._h is not None:
            check(lib().ntg_plan_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class gs_t:
    """gs_t%op(u, n, op) (sources/adjoint/adjoint_pnpn.f90:725)."""

    def __init__(self, coef: coef_t):
        self.coef = coef

    def op(self, u, op=GS_OP_ADD):
        if u.dtype == torch.float32:
            check(lib().ntg_gs_op_f32(self.coef.handle, _ptr(u, torch.float32, self.coef.n, "u"), int(op)))
        else:
            check(lib().ntg_gs_op(self.coef.handle, _ptr(u, n=self.coef.n, name="u"), int(op)))


class ax_helm_t:
    """Ax%compute(w, u, coef, msh, Xh) of ax_helm
    (sources/mapping_functions/PDE_filter_mapping.f90:177,256)."""

    def compute(self, w, u, coef: coef_t):
        if u.dtype == torch.float32:
            check(lib().ntg_ax_helm_f32(coef.handle, _ptr(w, torch.float32, coef.n, "w"),
                                        _ptr(u, torch.float32, coef.n, "u")))
        else:
            check(lib().ntg_ax_helm(coef.handle, _ptr(w, n=coef.n, name="w"), _ptr(u, n=coef.n, name="u")))


def bc_list_apply_scalar(coef: coef_t, x):
    if x.dtype == torch.float32:
        check(lib().ntg_bc_apply_scalar_f32(coef.handle, _ptr(x, torch.float32, coef.n, "x")))
    else:
        check(lib().ntg_bc_apply_scalar(coef.handle, _ptr(x, n=coef.n, name="x")))


class jacobi_t:
    """Jacobi pc_t: init(coef, dof, gs), update(), solve(z, r)
    (sources/mapping_functions/PDE_filter_mapping.f90:365-400)."""

    def __init__(self, coef: coef_t):
        self.coef = coef

    def update(self):
        check(lib().ntg_pc_jacobi_update(self.coef.handle))

    def solve(self, z, r):
        check(lib().ntg_pc_jacobi_solve(self.coef.handle, _ptr(z, n=self.coef.n, name="z"),
                                        _ptr(r, n=self.coef.n, name="r")))

    def dinv(self):
        d = torch.empty(self.coef.n, dtype=torch.float64, device=self.coef.device)
        check(lib().ntg_pc_jacobi_get(self.coef.handle, _ptr(d)))
        torch.cuda.synchronize()
        return d


class _ksp:
    def __init__(self, coef: coef_t, type_: int, max_iter: int, rtol: float, abstol: float):
        self.coef = coef
        h = C.c_void_p()
        check(lib().ntg_ksp_create(coef.handle, int(type_), int(max_iter), float(rtol), float(abstol), C.byref(h)))
        self._h = h
        self.type = type_
        self.max_iter = max_iter

    @property
    def handle(self):
        return self._h

    def set_inner(self, inner_rtol=1e-4, inner_max_iter=400):
        check(lib().ntg_ksp_set_inner(self._h, float(inner_rtol), int(inner_max_iter)))

    def set_restart(self, m):
        """GMRES restart length (1..31)."""
        check(lib().ntg_ksp_set_restart(self._h, int(m)))

    def set_check_every(self, k):
        check(lib().ntg_ksp_set_check_every(self._h, int(k)))

    def set_schwarz(self, sw):
        """Precondition with Schwarz (cg_mixed, gmres, gmres_mixed); None = Jacobi."""
        check(lib().ntg_ksp_set_schwarz(self._h, None if sw is None else sw.handle))
        self.sw = sw

    def set_tol(self, rtol, abstol):
        check(lib().ntg_ksp_set_tol(self._h, float(rtol), float(abstol)))

    def set_guess_guard(self, on=True):
        """Restart from zero when the initial guess's residual exceeds ||f||."""
        check(lib().ntg_ksp_set_guess_guard(self._h, int(bool(on))))

    def set_fused_update(self, on=True):
        """cg_mixed with a structured-box Schwarz: gather-scatter, mask and
        update of each iteration in one kernel (default) or three."""
        check(lib().ntg_ksp_set_fused_update(self._h, int(bool(on))))

    def solve(self, x, f) -> ksp_monitor_t:
        """ksp%solve(Ax, x, f, n, coef, blst, gs): x = guess in, solution out;
        f = assembled, masked RHS."""
        mon = ntg_monitor()
        check(lib().ntg_ksp_solve(self._h, _ptr(x, n=self.coef.n, name="x"), _ptr(f, n=self.coef.n, name="f"),
                                  C.byref(mon)))
        return ksp_monitor_t.from_c(mon)

    def solve_coupled(self, x, y, z, fx, fy, fz):
        mons = (ntg_monitor * 3)()
        n = self.coef.n
        check(lib().ntg_ksp_solve_coupled(self._h, _ptr(x, n=n), _ptr(y, n=n), _ptr(z, n=n), _ptr(fx, n=n),
                                          _ptr(fy, n=n), _ptr(fz, n=n), mons))
        return [ksp_monitor_t.from_c(m) for m in mons]

    def free(self):
        if self._h is not None:
            check(lib().ntg_ksp_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class schwarz_t:
    """Overlapping additive Schwarz preconditioner (FP32, fast-diagonalisation
    local solves).  With ``coarse=True`` it adds the coarse-grid correction
    on the element vertices (two-level Schwarz; the coarse part of Neko's
    'hsmg').  A structured box coef_t (coef_t.box) takes the box form
    (overlap across faces, edges and corners; separable coarse solve); any
    other mesh (coef_t.from_vertices, nmsh.coef_from_nmsh), or
    ``general=True``, the general form (overlap across the six faces, found
    through the global node ids; Galerkin coarse operator, at most 8192
    active vertices)."""

    def __init__(self, coef: coef_t, coarse: bool = False, general: bool | None = None):
        if general is None:
            general = not hasattr(coef, "box_dims")
        h = C.c_void_p()
        if general:
            check(lib().ntg_schwarz_create_general(coef.handle, _ptr(coef.x), _ptr(coef.y), _ptr(coef.z),
                                                   C.byref(h)))
        else:
            if not hasattr(coef, "box_dims"):
                raise ValueError("the box form of schwarz_t needs a structured box mesh (coef_t.box)")
            ex, ey, ez = coef.box_dims
            check(lib().ntg_schwarz_create(coef.handle, ex, ey, ez, _ptr(coef.x), _ptr(coef.y), _ptr(coef.z),
                                           C.byref(h)))
        self.general = bool(general)
        self._h = h
        self.coef = coef
        self.coarse = bool(coarse)
        if coarse:
            check(lib().ntg_schwarz_set_coarse(self._h, 1))

    @property
    def handle(self):
        return self._h

    def update(self):
        """Refresh the element means of h1/h2 after coef_t.set_coefs (and the
        coarse level's Dirichlet faces after coef_t.set_mask)."""
        check(lib().ntg_schwarz_update(self._h))

    def set_fdm_path(self, path=0):
        """FDM local solves: 0 (default) FP32 cores with even-odd transforms,
        1 tensor cores (lx = 8), 2 FP32 cores with full 1D products."""
        check(lib().ntg_schwarz_set_fdm_path(self._h, int(path)))

    def set_mass_term(self, enable: bool = True):
        """Add w D^-1 r (D the assembled diagonal, w the node's mass fraction):
        for mass terms varying inside elements (Brinkman penalisation)."""
        check(lib().ntg_schwarz_set_mass_term(self._h, int(bool(enable))))

    def apply(self, z, r):
        check(lib().ntg_schwarz_apply(self._h, _ptr(z, torch.float32, self.coef.n, "z"),
                                      _ptr(r, torch.float32, self.coef.n, "r")))

    def free(self):
        if self._h is not None:
            check(lib().ntg_schwarz_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def krylov_solver_factory(coef: coef_t, type_: str = "cg", max_iter: int = 800, rtol: float = 1e-10,
                          abstol: float = 0.0) -> _ksp:
    """krylov_solver_factory(ksp, n, type, max_iter, abstol)
    (sources/adjoint/adjoint_scheme.f90:1046-1055).  type: 'cg' (FP64
    Jacobi-PCG), 'cg_mixed' (FP32 PCG with FP64 reliable updates),
    'fcg_mixed' (FP32 inner PCG in an FP64 flexible CG), 'gmres' (FP64
    restarted flexible GMRES) or 'gmres_mixed' (FP32 GMRES cycles inside FP64
    iterative refinement)."""
    t = {"cg": KSP_CG, "fcg_mixed": KSP_FCG_MIXED, "cg_mixed": KSP_CG_MIXED, "gmres": KSP_GMRES,
         "gmres_mixed": KSP_GMRES_MIXED}.get(type_)
    if t is None:
        raise ValueError(f"unknown solver type {type_!r}")
    return _ksp(coef, t, max_iter, rtol, abstol)


def profiler_start_region(name: str, colour: int = 0):
    """Neko's profiler_start_region: an NVTX range named as the reference's
    regions are (e.g. 'Pressure solve')."""
    check(lib().ntg_profiler_start_region(name.encode(), int(colour)))


def profiler_end_region():
    check(lib().ntg_profiler_end_region())


class profiler_region:
    """with profiler_region('Pressure solve', 3): ... (start/end pair)."""

    def __init__(self, name: str, colour: int = 0):
        self.name, self.colour = name, colour

    def __enter__(self):
        profiler_start_region(self.name, self.colour)
        return self

    def __exit__(self, *a):
        profiler_end_region()


class projection_t:
    """Residual projection: init(n, L, activ_step), pre_solving(b, tstep),
    post_solving(x, tstep) (sources/adjoint/adjoint_pnpn.f90:365-374,729-741;
    projection_space_size 20 and projection_hold_steps 5 are the defaults at
    sources/adjoint/adjoint_scheme.f90:386-403).  With tstep given, steps up
    to activ_step neither project nor enter the basis; without it the
    projection is always active."""

    def __init__(self, coef: coef_t, L: int = 20, activ_step: int = 0):
        self.coef = coef
        h = C.c_void_p()
        check(lib().ntg_proj_create(coef.handle, int(L), C.byref(h)))
        self._h = h
        self.L = L
        self.activ_step = int(activ_step)
        self._active = True

    def _set_step(self, tstep):
        self._active = tstep is None or tstep > self.activ_step
        return self._active

    def pre_solving(self, b, tstep=None):
        if not self._set_step(tstep):
            return
        check(lib().ntg_proj_pre_solving(self._h, _ptr(b, n=self.coef.n, name="b")))

    def pre_solving_with(self, b, g):
        """pre_solving plus the extra direction g for this solve (learned guess)."""
        self._active = True
        used = C.c_int()
        check(lib().ntg_proj_pre_solving_with(self._h, _ptr(b, n=self.coef.n, name="b"),
                                              _ptr(g, n=self.coef.n, name="g"), C.byref(used)))
        return bool(used.value)

    def post_solving(self, x, tstep=None):
        if tstep is not None and tstep <= self.activ_step:
            return
        if not self._active:  # pre_solving was skipped for this solve
            return
        check(lib().ntg_proj_post_solving(self._h, _ptr(x, n=self.coef.n, name="x")))

    def record(self, b, x):
        """Enter a solution x of the (assembled, masked) right-hand side b
        that was found elsewhere, as pre_solving(b) + solve +
        post_solving would have; b and x are not modified."""
        check(lib().ntg_proj_pre_solving(self._h, _ptr(b.clone(), n=self.coef.n, name="b")))
        check(lib().ntg_proj_post_solving_full(self._h, _ptr(x, n=self.coef.n, name="x")))

    def state(self):
        """(m, xs [m, n], axs [m, n]): a copy of the basis and its A-images."""
        m = C.c_int()
        check(lib().ntg_proj_state(self._h, C.byref(m), None, None, 0))
        n = self.coef.n
        xs = torch.empty((m.value, n), dtype=torch.float64, device=self.coef.device)
        axs = torch.empty_like(xs)
        if m.value:
            check(lib().ntg_proj_state(self._h, C.byref(m), C.c_void_p(xs.data_ptr()), C.c_void_p(axs.data_ptr()),
                                       0))
        return m.value, xs, axs

    def load_state(self, m, xs, axs):
        mm = C.c_int(int(m))
        if m:
            xs = xs.to(device=self.coef.device, dtype=torch.float64).contiguous()
            axs = axs.to(device=self.coef.device, dtype=torch.float64).contiguous()
            check(lib().ntg_proj_state(self._h, C.byref(mm), C.c_void_p(xs.data_ptr()), C.c_void_p(axs.data_ptr()),
                                       1))
        else:
            check(lib().ntg_proj_state(self._h, C.byref(mm), None, None, 1))

    @property
    def size(self):
        return int(lib().ntg_proj_size(self._h))

    def reset(self):
        """Empty the basis (after the operator changed)."""
        self.free()
        h = C.c_void_p()
        check(lib().ntg_proj_create(self.coef.handle, int(self.L), C.byref(h)))
        self._h = h

    def free(self):
        if self._h is not None:
            check(lib().ntg_proj_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class learned_guess_t:
    """Per-element MLP initial guess, (history + 1) * 512 -> 64 -> 64 -> 512
    nodal correction of the newest solution, trained online on the solver's
    own solutions (tcgen05 BF16 tensor-core GEMMs, FP32 accumulate, Adam)."""

    def __init__(self, coef: coef_t, history=4, hidden=64, seed=0, lr=1e-3):
        self.coef = coef
        h = C.c_void_p()
        check(lib().ntg_guess_create(coef.handle, int(history), int(hidden), int(seed), C.byref(h)))
        self._h = h
        self.history, self.hidden = history, hidden
        self.F = (history + 1) * coef.lx ** 3
        self.O = coef.lx ** 3  # nodal output head
        check(lib().ntg_guess_set_lr(h, float(lr)))

    def predict(self, b, x):
        """Write the guess for rhs b into x; False until the history is full."""
        ready = C.c_int()
        check(lib().ntg_guess_predict(self._h, _ptr(b, n=self.coef.n), _ptr(x, n=self.coef.n), C.byref(ready)))
        return bool(ready.value)

    def observe(self, b, x, train_steps=0):
        loss = C.c_double()
        check(lib().ntg_guess_observe(self._h, _ptr(b, n=self.coef.n), _ptr(x, n=self.coef.n), int(train_steps),
                                      C.byref(loss)))
        return loss.value

    def reset_history(self):
        check(lib().ntg_guess_reset_history(self._h))

    def state(self):
        """Checkpoint: {'buf': FP32 device tensor, 'ints': [4], 'hrms': [8]}."""
        n = int(lib().ntg_guess_state_len(self._h))
        buf = torch.empty(n, dtype=torch.float32, device=self.coef.device)
        ints = (C.c_longlong * 4)()
        hrms = (C.c_double * 8)()
        check(lib().ntg_guess_state(self._h, C.c_void_p(buf.data_ptr()), ints, hrms, 0))
        return {"buf": buf, "ints": list(ints), "hrms": list(hrms)}

    def load_state(self, st):
        buf = st["buf"].to(device=self.coef.device, dtype=torch.float32).contiguous()
        if buf.numel() != int(lib().ntg_guess_state_len(self._h)):
            raise ValueError("network checkpoint of another shape")
        ints = (C.c_longlong * 4)(*[int(v) for v in st["ints"]])
        hrms = (C.c_double * 8)(*[float(v) for v in st["hrms"]])
        check(lib().ntg_guess_state(self._h, C.c_void_p(buf.data_ptr()), ints, hrms, 1))

    @property
    def num_params(self):
        return int(lib().ntg_guess_num_params(self._h))

    def get_params(self):
        p = torch.empty(self.num_params, dtype=torch.float32, device=self.coef.device)
        check(lib().ntg_guess_params(self._h, _ptr(p, torch.float32), 0))
        torch.cuda.synchronize()
        return p

    def set_params(self, p):
        check(lib().ntg_guess_params(self._h, _ptr(p, torch.float32, self.num_params, "params"), 1))

    # raw network access (X: int16 tensor of BF16 bit patterns, [E, F]; Y [E, 512])
    def forward_raw(self, Xbits, E):
        Y = torch.empty(E * self.O, dtype=torch.float32, device=self.coef.device)
        check(lib().ntg_guess_forward_raw(self._h, C.c_void_p(Xbits.data_ptr()), int(E), _ptr(Y, torch.float32)))
        torch.cuda.synchronize()
        return Y.view(E, self.O)

    def grad_raw(self, Xbits, T, E):
        g = torch.empty(self.num_params, dtype=torch.float32, device=self.coef.device)
        loss = C.c_double()
        check(lib().ntg_guess_grad_raw(self._h, C.c_void_p(Xbits.data_ptr()), _ptr(T, torch.float32), int(E),
                                       _ptr(g, torch.float32), C.byref(loss)))
        torch.cuda.synchronize()
        return loss.value, g

    def train_raw(self, Xbits, T, E):
        loss = C.c_double()
        check(lib().ntg_guess_train_raw(self._h, C.c_void_p(Xbits.data_ptr()), _ptr(T, torch.float32), int(E),
                                        C.byref(loss)))
        return loss.value

    def free(self):
        if self._h is not None:
            check(lib().ntg_guess_destroy(self._h))
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def ar1_modes(seed, nmodes, nsolves, rho=0.98, kmax=4):
    """Mode parameters of a right-hand-side sequence: integer wave vectors in
    [1, kmax]^3 and phases fixed per mode, amplitudes c_m(t)/|k_m|^2 with
    c_m an AR(1) process c(t+1) = rho c(t) + sqrt(1 - rho^2) eps (standard
    normal innovations, seeded).  Returns (k [3*nmodes], phases, amps
    [nsolves x nmodes])."""
    import numpy as np
    rng = np.random.default_rng(seed)
    k = rng.integers(1, kmax + 1, size=(nmodes, 3)).astype(np.int32)
    ph = rng.uniform(0, 2 * np.pi, nmodes)
    kk = (k.astype(np.float64) ** 2).sum(1)
    c = np.empty((nsolves, nmodes))
    c[0] = rng.standard_normal(nmodes)
    s = np.sqrt(1 - rho * rho)
    for t in range(1, nsolves):
        c[t] = rho * c[t - 1] + s * rng.standard_normal(nmodes)
    return k.ravel(), ph, c / kk


class SolveSequence:
    """Solve-sequence driver in the reference's order
    (sources/adjoint/adjoint_pnpn.f90:714-743): the caller's RHS is already
    gs-assembled and masked; then initial guess -> pc update -> ksp solve ->
    projection post / history update.  Guess modes:

      "zero"          x0 = 0
      "projection"    Fischer residual projection over the last L solutions
      "learned"       projection whose space is enriched, for this solve, by
                      the learned guess (Galerkin in the A-norm: never worse
                      than "projection")
      "learned_only"  the learned guess as x0, behind the ksp's guard (a guess
                      worse than zero is replaced by zero)

    Every solve converges to the same tolerance, relative to the original
    right-hand side, whatever the guess.  Each solve runs inside the
    profiler region `region` (the reference's 'Pressure solve',
    adjoint_pnpn.f90:733), and with `log` (a path or a writable file) each
    solve appends one JSON line: solve index, iterations, FP64 operator
    applications, start / final residual, right-hand-side norm, status,
    guess used and its wall time; the caller may add fields per solve
    (e.g. the error against an FP64 solution) through solve(f, extra=...).
    state_dict / load_state_dict checkpoint everything the next solve
    depends on (projection basis, network weights, Adam moments and step,
    solution history, counters), so a sequence resumes bit for bit."""

    def __init__(self, coef: coef_t, method="cg_mixed", guess="zero", rtol=1e-10, max_iter=50000, L=20,
                 history=4, hidden=64, seed=0, lr=1e-3, train_steps=20, pc="jacobi", delta=None, log=None,
                 region="Pressure solve", region_colour=3):
        if guess not in ("zero", "projection", "learned", "learned_only"):
            raise ValueError(f"unknown guess mode {guess!r}")
        if pc not in ("jacobi", "schwarz", "schwarz2"):
            raise ValueError(f"preconditioner {pc!r} is not built (jacobi, schwarz, schwarz2)")
        self.coef, self.guess, self.rtol = coef, guess, rtol
        self.ksp = krylov_solver_factory(coef, method, max_iter, rtol)
        self.sw = None
        if pc != "jacobi":
            if method != "cg_mixed":
                raise ValueError("the Schwarz preconditioner drives the cg_mixed solver")
            self.sw = schwarz_t(coef, coarse=pc == "schwarz2")
            self.ksp.set_schwarz(self.sw)
        if delta is not None:
            self.ksp.set_inner(delta, 1)
        self.proj = projection_t(coef, L) if guess in ("projection", "learned") else None
        self.net = learned_guess_t(coef, history, hidden, seed, lr) if guess.startswith("learned") else None
        if guess == "learned_only":
            self.ksp.set_guess_guard(True)
        self.train_steps = train_steps
        self.training = True
        self.nsolved = 0
        self.region, self.region_colour = region, region_colour
        self._log_own = isinstance(log, str)
        self._log = open(log, "a") if isinstance(log, str) else log
        self.x = torch.zeros(coef.n, dtype=torch.float64, device=coef.device)
        self.g = torch.zeros(coef.n, dtype=torch.float64, device=coef.device) if self.net is not None else None

    def solve(self, f, extra=None):
        """Returns (x, monitor, guess used, ||f||)."""
        import time
        t0 = time.perf_counter() if self._log is not None else 0.0
        x = self.x
        x.zero_()
        used = "zero"
        fn = glsc3(self.coef, f, f, self._mult()) ** 0.5
        profiler_start_region(self.region, self.region_colour)
        try:
            if self.proj is not None:
                # the reduced system keeps the tolerance of the original RHS
                b = f.clone()
                used = "projection"
                if self.net is not None and self.net.predict(f, self.g):
                    if self.proj.pre_solving_with(b, self.g):
                        used = "projection+learned"
                else:
                    self.proj.pre_solving(b)
                self.ksp.set_tol(0.0, self.rtol * fn)
                mon = self.ksp.solve(x, b)
                self.proj.post_solving(x)
            else:
                if self.net is not None and self.net.predict(f, x):
                    used = "learned"
                mon = self.ksp.solve(x, f)
                if mon.guess_rejected:
                    used = "zero (learned rejected)"
            if self.net is not None:
                self.net.observe(f, x, self.train_steps if self.training else 0)
        finally:
            profiler_end_region()
        if self._log is not None:
            import json
            torch.cuda.synchronize(self.coef.device)
            rec = {"solve": self.nsolved, "iter": mon.iter, "inner_iter": mon.inner_iter, "fp64_ax": mon.fp64_ax,
                   "res_start": mon.res_start, "res_final": mon.res_final, "rhs_norm": fn,
                   "rel_res": mon.res_final / fn if fn > 0 else 0.0, "status": mon.status, "guess": used,
                   "training": bool(self.training and self.net is not None),
                   "time_s": round(time.perf_counter() - t0, 6)}
            if extra:
                rec.update(extra)
            self._log.write(json.dumps(rec) + "\n")
            self._log.flush()
        self.nsolved += 1
        return x, mon, used, fn

    def record(self, f, x):
        """Take a converged solution x of f found elsewhere (another solver,
        a restart) into the guess state, as if this sequence had solved it:
        the projection basis and the network's history are updated; nothing
        is solved."""
        if self.proj is not None:
            self.proj.record(f, x)
        if self.net is not None:
            self.net.observe(f, x, 0)
        self.nsolved += 1

    def coefficients_changed(self):
        """Refresh what depends on h1/h2 (Jacobi diagonal, Schwarz means)
        after coef_t.set_coefs; the projection basis is restarted, since its
        A-conjugacy belonged to the old operator."""
        if self.sw is not None:
            self.sw.update()
        if self.proj is not None:
            self.proj.reset()

    def state_dict(self):
        """Everything the next solve depends on, as host tensors."""
        st = {"nsolved": self.nsolved, "training": self.training, "guess": self.guess}
        if self.proj is not None:
            m, xs, axs = self.proj.state()
            st["proj"] = {"m": m, "xs": xs.cpu(), "axs": axs.cpu()}
        if self.net is not None:
            st["net"] = {k: (v.cpu() if isinstance(v, torch.Tensor) else v) for k, v in self.net.state().items()}
        return st

    def load_state_dict(self, st):
        if st["guess"] != self.guess:
            raise ValueError(f"checkpoint of guess mode {st['guess']!r}, sequence is {self.guess!r}")
        self.nsolved, self.training = int(st["nsolved"]), bool(st["training"])
        if self.proj is not None:
            p = st["proj"]
            self.proj.load_state(p["m"], p["xs"], p["axs"])
        if self.net is not None:
            self.net.load_state(st["net"])

    def save(self, path):
        torch.save(self.state_dict(), path)

    def load(self, path):
        self.load_state_dict(torch.load(path, map_location="cpu", weights_only=False))

    def close(self):
        if self._log is not None and self._log_own:
            self._log.close()
        self._log = None

    def _mult(self):
        if not hasattr(self, "_mult_t"):
            self._mult_t = self.coef.geometry()["mult"]
        return self._mult_t


def glsc3(coef: coef_t, a, b, c=None) -> float:
    out = C.c_double()
    n = a.numel()
    check(lib().ntg_glsc3(coef.handle, _ptr(a, n=n), _ptr(b, n=n), _ptr(c, n=n) if c is not None else None, n,
                          C.byref(out)))
    return out.value


class RAMP_mapping_t:
    """RAMP mapping (sources/mapping_functions/RAMP_mapping.f90:101-267);
    defaults of RAMP_mapping_init_from_json (f_min 0, f_max 1000, q 1,
    convex_up)."""

    def __init__(self, f_min=0.0, f_max=1000.0, q=1.0, convex_up=True):
        self.f_min, self.f_max, self.q, self.convex_up = f_min, f_max, q, convex_up

    def apply_forward(self, X_out, X_in):
        check(lib().ntg_ramp_forward(_ptr(X_out), _ptr(X_in), X_in.numel(), self.f_min, self.f_max, self.q,
                                     int(self.convex_up), _stream()))

    def apply_backward(self, dF_dX_in, dF_dX_out, X_in):
        check(lib().ntg_ramp_backward(_ptr(dF_dX_in), _ptr(dF_dX_out), _ptr(X_in), X_in.numel(), self.f_min,
                                      self.f_max, self.q, int(self.convex_up), _stream()))


class PDE_filter_t:
    """PDE density filter (sources/mapping_functions/PDE_filter_mapping.f90:126-363):
    (r^2 K + B) X_out = B X_in, all-Neumann, initial guess X_in; r = 0.01,
    abstol 1e-10, 200 iterations by default."""

    def __init__(self, coef: coef_t, r=0.01, abstol=1e-10, max_iter=200, log=None):
        self.coef, self.r = coef, r
        self.ksp = krylov_solver_factory(coef, "cg", max_iter, 0.0, abstol)
        self.ksp_results = None
        self.log = log  # None, or a callable taking each solve's log line

    def _apply(self, X_out, X_in):
        mon = ntg_monitor()
        # the solve inside the reference's 'filter solve' region
        # (PDE_filter_mapping.f90:254-259)
        with profiler_region("filter solve"):
            check(lib().ntg_filter_apply(self.coef.handle, self.ksp.handle, _ptr(X_out, n=self.coef.n),
                                         _ptr(X_in, n=self.coef.n), float(self.r), C.byref(mon)))
        self.ksp_results = ksp_monitor_t.from_c(mon)
        if self.log is not None:
            # the reference's 'Filter' message (PDE_filter_mapping.f90:264-272)
            m = self.ksp_results
            self.log("Filter\nIterations:   Start residual:     Final residual:\n"
                     f"{m.iter:11d}   {m.res_start:15.7E}     {m.res_final:15.7E}")
        return self.ksp_results

    def apply_forward(self, X_out, X_in):
        return self._apply(X_out, X_in)

    def apply_backward(self, dF_dX_in, dF_dX_out, X_in=None):
        return self._apply(dF_dX_in, dF_dX_out)


class simple_brinkman_source_term_t:
    """f -= chi * u per component
    (sources/source_terms/simple_brinkman_source_term.f90:139-153)."""

    def __init__(self, fx, fy, fz, u, v, w, chi):
        self.fields = (fx, fy, fz)
        self.u, self.v, self.w, self.chi = u, v, w, chi

    def compute(self, t=0.0, tstep=0, mask=None, base=1):
        fx, fy, fz = self.fields
        check(lib().ntg_brinkman_compute(_ptr(fx), _ptr(fy), _ptr(fz), _ptr(self.u), _ptr(self.v), _ptr(self.w),
                                         _ptr(self.chi), fx.numel(), _ptr(mask, torch.int32) if mask is not None
                                         else None, 0 if mask is None else mask.numel(), int(base), _stream()))


def permeability(kappa, phi, perm0, perm1, penalty):
    """design_t%update_permeability (sources/topology_optimization/design.f90:316-348)."""
    check(lib().ntg_permeability(_ptr(kappa), _ptr(phi), phi.numel(), float(perm0), float(perm1), float(penalty),
                                 _stream()))


def sens_min_dissipation(s, u, v, w, ua, va, wa, if_lube=False, K_scale=0.0):
    check(lib().ntg_sens_min_dissipation(_ptr(s), _ptr(u), _ptr(v), _ptr(w), _ptr(ua), _ptr(va), _ptr(wa), u.numel(),
                                         int(bool(if_lube)), float(K_scale), _stream()))


# derivative operators, Neko's operators.f90 as the adjoint terms call them
# (sources/adjoint/adv_adjoint_no_dealias.f90, FP64, on the current stream)
_DIRS = {"x": 0, "y": 1, "z": 2, 0: 0, 1: 1, 2: 2}


def _f(coef, t, name):
    return _ptr(t, n=coef.n, name=name)


def opgrad(ux, uy, uz, u, coef: coef_t):
    """(ux, uy, uz) = B grad u (weak gradient)."""
    check(lib().ntg_opgrad(coef.metrics().handle, _f(coef, ux, "ux"), _f(coef, uy, "uy"), _f(coef, uz, "uz"),
                           _f(coef, u, "u")))


def dudxyz(du, u, direction, coef: coef_t):
    """du = du/dx_direction (strong), direction "x" | "y" | "z"."""
    check(lib().ntg_dudxyz(coef.metrics().handle, _f(coef, du, "du"), _f(coef, u, "u"), _DIRS[direction]))


def cdtp(dtx, x, direction, coef: coef_t):
    """dtx = transpose of opgrad's `direction` component applied to x
    (Neko's cdtp(dtx, x, dr, ds, dt, coef) with the direction's cofactors)."""
    check(lib().ntg_cdtp(coef.metrics().handle, _f(coef, dtx, "dtx"), _f(coef, x, "x"), _DIRS[direction]))


def conv1(du, u, vx, vy, vz, coef: coef_t):
    """du = (v . grad) u (strong, pointwise)."""
    check(lib().ntg_conv1(coef.metrics().handle, _f(coef, du, "du"), _f(coef, u, "u"), _f(coef, vx, "vx"),
                          _f(coef, vy, "vy"), _f(coef, vz, "vz")))


def curl(w1, w2, w3, u1, u2, u3, coef: coef_t):
    """w = Binv gs(B curl u)."""
    check(lib().ntg_curl(coef.metrics().handle, *[_f(coef, t, f"w{i}") for i, t in enumerate((w1, w2, w3))],
                         *[_f(coef, t, f"u{i}") for i, t in enumerate((u1, u2, u3))]))


@dataclass
class solver_config_t:
    """Solver wiring of one field as the reference reads it from the case
    file (sources/adjoint/adjoint_scheme.f90:693-851): Krylov type,
    preconditioner, absolute tolerance, iteration cap, projection space."""
    field: str
    ksp: str
    pc: str
    abstol: float
    max_iter: int
    projection_space_size: int
    projection_hold_steps: int


def load_case(text):
    """Parse a Neko case file: JSON with // comments and trailing commas
    (outside strings)."""
    import json

    def strip(src, drop):
        out, i, n, in_str = [], 0, len(src), False
        while i < n:
            ch = src[i]
            if in_str:
                out.append(ch)
                if ch == "\\" and i + 1 < n:
                    out.append(src[i + 1])
                    i += 1
                elif ch == '"':
                    in_str = False
            elif ch == '"':
                in_str = True
                out.append(ch)
            else:
                k = drop(src, i)
                if k > i:
                    i = k
                    continue
                out.append(ch)
            i += 1
        return "".join(out)

    def comment(src, i):  # "//" to the end of the line
        if src.startswith("//", i):
            j = src.find("\n", i)
            return len(src) if j < 0 else j
        return i

    def trailing_comma(src, i):  # a comma before a closing bracket
        if src[i] == ",":
            j = i + 1
            while j < len(src) and src[j] in " \t\r\n":
                j += 1
            if j < len(src) and src[j] in "}]":
                return i + 1
        return i

    return json.loads(strip(strip(text, comment), trailing_comma))


def solver_from_case(params, field="pressure"):
    """The reference's lookup for the pressure or velocity solver: the key
    under case.adjoint falls back to case.fluid; max_iterations defaults to
    800, projection_space_size to 20 and projection_hold_steps to 5
    (adjoint_scheme.f90:386-403, 693-851)."""
    if field not in ("pressure", "velocity"):
        raise ValueError("field is 'pressure' or 'velocity'")
    case = params.get("case", params)

    def get(key, default=None, required=False):
        for section in ("adjoint", "fluid"):
            v = case.get(section, {}).get(f"{field}_solver", {}).get(key)
            if v is not None:
                return v
        if required:
            raise KeyError(f"case.fluid.{field}_solver.{key} is required")
        return default

    # the projection keys are read only under <field>_solver, as the
    # reference does (adjoint_scheme.f90:384-403); a key placed directly
    # under case.adjoint or case.fluid is ignored
    return solver_config_t(field, str(get("type", required=True)), str(get("preconditioner", required=True)),
                           float(get("absolute_tolerance", required=True)), int(get("max_iterations", 800)),
                           int(get("projection_space_size", 20)), int(get("projection_hold_steps", 5)))


_KSP_FAST = {"cg": "cg_mixed", "gmres": "gmres_mixed"}


def build_solver(coef: coef_t, cfg: solver_config_t, fast=True):
    """Krylov solver and preconditioner for a case's solver entry.  fast:
    the FP32-inner variants ("cg" -> cg_mixed, "gmres" -> gmres_mixed) at the
    same absolute tolerance; "hsmg" maps to the two-level Schwarz, "jacobi"
    to Jacobi.  Returns (ksp, projection or None)."""
    if cfg.ksp not in ("cg", "gmres"):
        raise ValueError(f"solver type {cfg.ksp!r} is not built (cg, gmres)")
    if cfg.pc not in ("jacobi", "hsmg"):
        raise ValueError(f"preconditioner {cfg.pc!r} is not built (jacobi, hsmg)")
    kind = _KSP_FAST[cfg.ksp] if fast else cfg.ksp
    ksp = krylov_solver_factory(coef, kind, cfg.max_iter, 0.0, cfg.abstol)
    if cfg.pc == "hsmg":
        ksp.set_schwarz(schwarz_t(coef, coarse=True))
        if kind == "cg_mixed":
            ksp.set_inner(2.2e-4, 1)  # reliable-update spacing measured for the two-level Schwarz
    proj = projection_t(coef, cfg.projection_space_size, cfg.projection_hold_steps) \
        if cfg.projection_space_size > 0 else None
    return ksp, proj


class pnpn_step_t:
    """The solve sequence of one Pn/Pn step in the reference's order
    (sources/adjoint/adjoint_pnpn.f90:714-801):

      pressure  prs_res -> gs -> bc -> projection pre -> pc update + solve
                (zero initial guess) -> projection post -> p += dp
      velocity  vel_res -> gs (3 components) -> bc -> projection pre ->
                coupled solve -> projection post -> u += du

    Two coef_t of the same mesh carry the pressure operator (h1 = 1/rho, no
    mass term, its Dirichlet mask) and the velocity operator (h1 = mu,
    h2 = rho bd/dt, its Dirichlet mask, shared by the three components).
    L = 0 switches the projections off; activ_step is the reference's
    projection_hold_steps.  With projection each solve is held to rtol times
    the norm of its unprojected right-hand side (an absolute tolerance, as
    the reference's solvers use), and the velocity components are solved one
    after another."""

    def __init__(self, coef_p: coef_t, coef_v: coef_t, prs_solver="cg", vel_solver="cg", max_iter=800,
                 rtol=1e-10, L=20, activ_step=5):
        self.cp, self.cv = coef_p.metrics(), coef_v.metrics()
        self.ksp_p = krylov_solver_factory(coef_p, prs_solver, max_iter, rtol)
        self.ksp_v = krylov_solver_factory(coef_v, vel_solver, max_iter, rtol)
        self.proj_p = projection_t(coef_p, L, activ_step) if L else None
        self.proj_v = [projection_t(coef_v, L, activ_step) for _ in range(3)] if L else None
        self.prs, self.vel = pnpn_prs_res_t(), pnpn_vel_res_t()
        self.gs_p, self.gs_v = gs_t(coef_p), gs_t(coef_v)
        self.rtol = float(rtol)
        self.mult = coef_p.geometry()["mult"] if L else None
        z = lambda: torch.zeros(coef_p.n, dtype=torch.float64, device=coef_p.device)
        self.p_res, self.dp = z(), z()
        self.res = [z() for _ in range(3)]
        self.du = [z() for _ in range(3)]

    @staticmethod
    def _inv(v):
        return 1.0 / v if isinstance(v, torch.Tensor) else 1.0 / float(v)

    def step(self, u, v, w, p, ue, ve, we, fx, fy, fz, mu=1.0, rho=1.0, bd=1.0, dt=1.0, tstep=None,
             prs_surface=None, sym_surface=None, base=1):
        """Advances p and (u, v, w) in place; returns the pressure monitor
        and the three velocity monitors."""
        cp, cv = self.cp, self.cv
        # profiler regions and colours as the reference names them
        # (adjoint_pnpn.f90:715,733,746,783)
        profiler_start_region("Pressure residual", 18)
        self.prs.compute(p, self.p_res, u, v, w, ue, ve, we, fx, fy, fz, cp, prs_surface, sym_surface, bd=bd,
                         dt=dt, mu=mu, rho=rho, base=base)
        self.gs_p.op(self.p_res)
        bc_list_apply_scalar(cp, self.p_res)
        profiler_end_region()
        h1p = self._inv(rho)
        if isinstance(h1p, torch.Tensor):
            cp.set_coefs(h1=h1p.contiguous(), ifh2=False)
        else:
            cp.set_coefs(h1c=h1p, ifh2=False)
        if self.proj_p is not None:
            # the projected system keeps the tolerance of the original
            # right-hand side (the reference's absolute tolerance)
            self.ksp_p.set_tol(0.0, self.rtol * glsc3(cp, self.p_res, self.p_res, self.mult) ** 0.5)
            self.proj_p.pre_solving(self.p_res, tstep)
        self.dp.zero_()
        with profiler_region("Pressure solve", 3):
            mon_p = self.ksp_p.solve(self.dp, self.p_res)
        if self.proj_p is not None:
            self.proj_p.post_solving(self.dp, tstep)
        p.add_(self.dp)
        profiler_start_region("Velocity residual", 19)
        self.vel.compute(u, v, w, *self.res, p, fx, fy, fz, cv, mu=mu, rho=rho, bd=bd, dt=dt)
        for r in self.res:
            self.gs_v.op(r)
            bc_list_apply_scalar(cv, r)
        profiler_end_region()
        h2v = (rho * (bd / dt)) if isinstance(rho, torch.Tensor) else torch.full_like(self.dp, float(rho) * bd / dt)
        if isinstance(mu, torch.Tensor):
            cv.set_coefs(h1=mu.contiguous(), h2=h2v.contiguous(), ifh2=True)
        else:
            cv.set_coefs(h1c=float(mu), h2=h2v.contiguous(), ifh2=True)
        for d in self.du:
            d.zero_()
        if self.proj_v is None:
            with profiler_region("Velocity solve", 4):
                mons_v = self.ksp_v.solve_coupled(*self.du, *self.res)
        else:
            # per component, each to the tolerance of its unprojected RHS
            mons_v = []
            for pr, r, d in zip(self.proj_v, self.res, self.du):
                self.ksp_v.set_tol(0.0, self.rtol * glsc3(cv, r, r, self.mult) ** 0.5)
                pr.pre_solving(r, tstep)
                with profiler_region("Velocity solve", 4):
                    mons_v.append(self.ksp_v.solve(d, r))
                pr.post_solving(d, tstep)
        for x, d in zip((u, v, w), self.du):
            x.add_(d)
        return mon_p, mons_v


class adv_lin_no_dealias_t:
    """Adjoint and linearised advection without dealiasing
    (sources/adjoint/adv_adjoint_no_dealias.f90: adjoint_advection_no_dealias
    :118-255 and linear_advection_no_dealias :365-427), same argument order:
    (vx, vy, vz) the adjoint / perturbation velocity, (vxb, vyb, vzb) the
    base flow, (fx, fy, fz) the right-hand side, updated in place."""

    def __init__(self, coef: coef_t):
        self.coef = coef.metrics()

    def compute_adjoint(self, vx, vy, vz, vxb, vyb, vzb, fx, fy, fz):
        c = self.coef
        check(lib().ntg_adjoint_advection_no_dealias(
            c.handle, *[_f(c, t, "f") for t in (fx, fy, fz)], *[_f(c, t, "v") for t in (vx, vy, vz)],
            *[_f(c, t, "vb") for t in (vxb, vyb, vzb)]))

    def compute_linear(self, vx, vy, vz, vxb, vyb, vzb, fx, fy, fz):
        c = self.coef
        check(lib().ntg_linear_advection_no_dealias(
            c.handle, *[_f(c, t, "f") for t in (fx, fy, fz)], *[_f(c, t, "v") for t in (vx, vy, vz)],
            *[_f(c, t, "vb") for t in (vxb, vyb, vzb)]))


class adv_lin_dealias_t:
    """Dealiased adjoint and linearised advection
    (sources/adjoint/adv_adjoint_dealias.f90: init_dealias :137-224,
    compute_adjoint :235-462, compute_linear :470-600), same argument order
    as adv_lin_no_dealias_t.  lxd None: 3 lx / 2 Gauss-Legendre points per
    direction (advection_adjoint_fctry.f90:66-90)."""

    def __init__(self, coef: coef_t, lxd=None):
        self.coef = coef.metrics()
        h = C.c_void_p()
        check(lib().ntg_dealias_create(C.byref(h), coef.handle, int(lxd or 0)))
        self._h = h
        l, ng = C.c_int(), C.c_int64()
        check(lib().ntg_dealias_info(h, C.byref(l), C.byref(ng)))
        self.lxd, self.n_gl = l.value, ng.value

    def map_to_gl(self, out_gl, x):
        check(lib().ntg_dealias_map(self._h, _ptr(out_gl, n=self.n_gl, name="out"), _f(self.coef, x, "x"), 1))

    def map_to_gll(self, out, x_gl):
        check(lib().ntg_dealias_map(self._h, _f(self.coef, out, "out"), _ptr(x_gl, n=self.n_gl, name="x"), 0))

    def _run(self, fn, vx, vy, vz, vxb, vyb, vzb, fx, fy, fz):
        c = self.coef
        check(fn(self._h, *[_f(c, t, "f") for t in (fx, fy, fz)], *[_f(c, t, "v") for t in (vx, vy, vz)],
                 *[_f(c, t, "vb") for t in (vxb, vyb, vzb)]))

    def compute_adjoint(self, vx, vy, vz, vxb, vyb, vzb, fx, fy, fz):
        self._run(lib().ntg_adjoint_advection_dealias, vx, vy, vz, vxb, vyb, vzb, fx, fy, fz)

    def compute_linear(self, vx, vy, vz, vxb, vyb, vzb, fx, fy, fz):
        self._run(lib().ntg_linear_advection_dealias, vx, vy, vz, vxb, vyb, vzb, fx, fy, fz)

    def free(self):
        if getattr(self, "_h", None) is not None:
            lib().ntg_dealias_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class adjoint_minimum_dissipation_source_term_t:
    """f += obj_scale curl(curl(u)), optionally kept inside a zone
    (sources/source_terms/adjoint_minimum_dissipation_source_term.f90:175-249;
    the zone is the point-zone mask, unique 1-based indices by default)."""

    def __init__(self, fields, u, v, w, coef: coef_t, obj_scale=1.0, mask=None, base=1):
        self.fields, self.u, self.v, self.w = tuple(fields), u, v, w
        self.coef, self.obj_scale, self.mask, self.base = coef.metrics(), float(obj_scale), mask, int(base)

    def compute(self, t=0.0, tstep=0):
        c, (fx, fy, fz) = self.coef, self.fields
        m = self.mask
        check(lib().ntg_adjoint_min_dissipation(
            c.handle, _f(c, fx, "fx"), _f(c, fy, "fy"), _f(c, fz, "fz"), _f(c, self.u, "u"), _f(c, self.v, "v"),
            _f(c, self.w, "w"), self.obj_scale, _ptr(m, torch.int32, name="mask") if m is not None else None,
            0 if m is None else m.numel(), self.base))


def _prop(coef, v, name):
    """(pointer, constant) of a material property given as a field or a number."""
    if isinstance(v, torch.Tensor):
        return _f(coef, v, name), 0.0
    return None, float(v)


def _surface(coef, surf, name):
    if surf is None:
        return None, None, 0
    idx, sv = surf
    if sv.shape != (3, idx.numel()):
        raise ValueError(f"{name}: s must be 3 x {idx.numel()} (normal times area per entry)")
    return _ptr(idx, torch.int32, name=name + " idx"), _ptr(sv.contiguous(), name=name + " s"), idx.numel()


class pnpn_prs_res_t:
    """Pressure residual of the Pn/Pn splitting, prs_res%compute
    (sources/adjoint/adjoint_pnpn.f90:716-723), same argument order.  The
    surface terms are (idx, s) pairs: unique node indices (base `base`, 1 for
    Neko masks) and s = 3 x len(idx) outward normals times facet areas.
    mu and rho are numbers or fields.  p_res is neither assembled nor masked."""

    def compute(self, p, p_res, u, v, w, u_e, v_e, w_e, f_x, f_y, f_z, c_Xh: coef_t, bc_prs_surface=None,
                bc_sym_surface=None, bd=1.0, dt=1.0, mu=1.0, rho=1.0, base=1):
        c = c_Xh.metrics()
        mp, mc = _prop(c, mu, "mu")
        rp, rc = _prop(c, rho, "rho")
        pi, ps, pn = _surface(c, bc_prs_surface, "bc_prs_surface")
        si, ss, sn = _surface(c, bc_sym_surface, "bc_sym_surface")
        check(lib().ntg_pnpn_prs_res(c.handle, _f(c, p_res, "p_res"), _f(c, p, "p"),
                                     *[_f(c, t, "u") for t in (u, v, w)], *[_f(c, t, "u_e") for t in (u_e, v_e, w_e)],
                                     *[_f(c, t, "f") for t in (f_x, f_y, f_z)], mp, mc, rp, rc, float(bd), float(dt),
                                     pi, ps, pn, si, ss, sn, int(base)))


class pnpn_vel_res_t:
    """Velocity residual of the Pn/Pn splitting, vel_res%compute
    (sources/adjoint/adjoint_pnpn.f90:747-753): u_res_c = f_c - (mu K +
    rho bd/dt B) u_c - B grad_c p, all three components in one pass; the
    coef's own h1/h2 are left as they were."""

    def compute(self, u, v, w, u_res, v_res, w_res, p, f_x, f_y, f_z, c_Xh: coef_t, mu=1.0, rho=1.0, bd=1.0,
                dt=1.0):
        c = c_Xh.metrics()
        mp, mc = _prop(c, mu, "mu")
        rp, rc = _prop(c, rho, "rho")
        check(lib().ntg_pnpn_vel_res(c.handle, *[_f(c, t, "res") for t in (u_res, v_res, w_res)],
                                     *[_f(c, t, "u") for t in (u, v, w)], _f(c, p, "p"),
                                     *[_f(c, t, "f") for t in (f_x, f_y, f_z)], mp, mc, rp, rc, float(bd), float(dt)))


def _hostvec(v, m, name):
    import numpy as np
    a = np.ascontiguousarray(np.broadcast_to(np.asarray(v, dtype=np.float64), (m,)))
    return a, a.ctypes.data_as(C.POINTER(C.c_double))


class mma_t:
    """The MMA optimiser on the GPU (sources/mma/mma.f90: init :186-295,
    update :297-324, KKT :355-393), same argument meaning: x, xmin, xmax,
    df0dx are CUDA tensors of n; fval has m values; dfdx is (m, n) as the
    reference stores it, i.e. a CUDA tensor whose entry (i, j) sits at
    i + m j (a torch tensor of shape (n, m), or of m * n entries)."""

    def __init__(self, x, n, m, a0, a, c, d, xmin, xmax, max_iter=None, epsimin=None, asyinit=None, asyincr=None,
                 asydecr=None):
        self.n, self.m = int(n), int(m)
        self._keep = [_hostvec(v, self.m, k) for k, v in (("a", a), ("c", c), ("d", d))]
        xmin = xmin if isinstance(xmin, torch.Tensor) else torch.full_like(x, float(xmin))
        xmax = xmax if isinstance(xmax, torch.Tensor) else torch.full_like(x, float(xmax))
        h = C.c_void_p()
        check(lib().ntg_mma_create(C.byref(h), self.n, self.m, _ptr(x, n=self.n, name="x"), float(a0),
                                   *[k[1] for k in self._keep], _ptr(xmin.contiguous(), n=self.n, name="xmin"),
                                   _ptr(xmax.contiguous(), n=self.n, name="xmax"), int(max_iter or 0),
                                   float(epsimin or 0.0), float(asyinit or 0.0), float(asyincr or 0.0),
                                   float(asydecr or 0.0), _stream()))
        self._h = h

    def _dfdx(self, dfdx):
        return _ptr(dfdx.contiguous(), n=self.n * self.m, name="dfdx")

    def update(self, iter, x, df0dx, fval, dfdx):
        fv, fp = _hostvec(fval, self.m, "fval")
        check(lib().ntg_mma_update(self._h, int(iter), _ptr(x, n=self.n, name="x"),
                                   _ptr(df0dx, n=self.n, name="df0dx"), fp, self._dfdx(dfdx)))

    def KKT(self, x, df0dx, fval, dfdx):
        fv, fp = _hostvec(fval, self.m, "fval")
        mx, nr = C.c_double(), C.c_double()
        check(lib().ntg_mma_kkt(self._h, _ptr(x, n=self.n, name="x"), _ptr(df0dx, n=self.n, name="df0dx"), fp,
                                self._dfdx(dfdx), C.byref(mx), C.byref(nr)))
        return mx.value, nr.value

    def _info(self):
        k, mx, nr = (C.c_longlong * 3)(), C.c_double(), C.c_double()
        check(lib().ntg_mma_info(self._h, k, C.byref(mx), C.byref(nr)))
        return tuple(k), mx.value, nr.value

    @property
    def residumax(self):
        return self._info()[1]

    @property
    def residunorm(self):
        return self._info()[2]

    @property
    def newton_steps(self):
        return self._info()[0][0]

    @property
    def counts(self):
        """(Newton steps, line-search trials, epsilon levels) so far."""
        return self._info()[0]

    def free(self):
        if getattr(self, "_h", None) is not None:
            lib().ntg_mma_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


class fld_file_t:
    """Field files in the Nek5000 binary format, as Neko's fld_file_t writes
    them for fld_file_output_t (sources/topology_optimization/
    topopt_design.f90:283-286): write(fields, t, tstep) and read().  Fields
    are CUDA tensors or numpy arrays of n = nelv lx^3 doubles, keyed x, y, z
    (coordinates), u, v, w (velocity), p, t (temperature) and s (a list of
    scalars).  precision "sp" writes float32 data (Neko's default), "dp"
    float64."""

    KEYS = ("x", "y", "z", "u", "v", "w", "p", "t")

    def __init__(self, fname, precision="sp"):
        if precision not in ("sp", "dp"):
            raise ValueError("precision is 'sp' or 'dp'")
        self.fname, self.wdsize = str(fname), 4 if precision == "sp" else 8

    @staticmethod
    def _arg(a):
        import numpy as np
        if a is None:
            return None, None
        if isinstance(a, torch.Tensor):
            if a.dtype != torch.float64 or not a.is_contiguous():
                raise TypeError("fields must be contiguous float64")
            return C.c_void_p(a.data_ptr()), (1 if a.is_cuda else 0)
        a = np.ascontiguousarray(a, dtype=np.float64)
        return C.c_void_p(a.ctypes.data), 0

    def write(self, fields, lx, nelv, t=0.0, tstep=0, glb_el=None):
        import numpy as np
        keep, ptrs, dev = [], [], set()
        for k in self.KEYS:
            a = fields.get(k)
            if a is not None and not isinstance(a, torch.Tensor):
                a = np.ascontiguousarray(a, dtype=np.float64)
            keep.append(a)
            pa, d = self._arg(a)
            ptrs.append(pa)
            if d is not None:
                dev.add(d)
        sc = [a if isinstance(a, torch.Tensor) else np.ascontiguousarray(a, dtype=np.float64)
              for a in fields.get("s", [])]
        sp = [self._arg(a) for a in sc]
        dev.update(d for _, d in sp)
        if len(dev) > 1:
            raise ValueError("fields must be all on the device or all on the host")
        sarr = (C.c_void_p * max(1, len(sp)))(*[p for p, _ in sp])
        el = None
        if glb_el is not None:
            el = np.ascontiguousarray(glb_el, dtype=np.int64)
        check(lib().ntg_fld_write(self.fname.encode(), int(lx), int(nelv),
                                  None if el is None else C.c_void_p(el.ctypes.data), float(t), int(tstep),
                                  self.wdsize, dev.pop() if dev else 0, *ptrs, sarr if sp else None, len(sp)))

    @staticmethod
    def write_index(path, name, first, count):
        """The "<name>.nek5000" file that visualisation tools open."""
        check(lib().ntg_fld_write_index(str(path).encode(), str(name).encode(), int(first), int(count)))

    def info(self):
        lx, ne, wd, st = C.c_int(), C.c_int64(), C.c_int(), C.c_int()
        tm = C.c_double()
        code = C.create_string_buffer(64)
        check(lib().ntg_fld_info(self.fname.encode(), C.byref(lx), C.byref(ne), C.byref(wd), C.byref(tm),
                                 C.byref(st), code, 64))
        return {"lx": lx.value, "nelv": ne.value, "wdsize": wd.value, "time": tm.value, "tstep": st.value,
                "rdcode": code.value.decode()}

    def read(self, device=None):
        """Dict of the fields the file holds (numpy arrays, or CUDA tensors on
        `device`) plus "glb_el" and the header items."""
        import numpy as np
        h = self.info()
        n = h["nelv"] * h["lx"] ** 3
        code = h["rdcode"]
        want = {"x": "X", "y": "X", "z": "X", "u": "U", "v": "U", "w": "U", "p": "P", "t": "T"}
        mk = (lambda: torch.empty(n, dtype=torch.float64, device=device)) if device is not None else \
            (lambda: np.empty(n))
        out = {k: mk() for k, c in want.items() if c in code}
        ns = int(code[code.index("S") + 1:code.index("S") + 3]) if "S" in code else 0
        out["s"] = [mk() for _ in range(ns)]
        el = np.empty(h["nelv"], dtype=np.int64)
        ptr = lambda a: None if a is None else C.c_void_p(a.data_ptr() if isinstance(a, torch.Tensor)
                                                           else a.ctypes.data)
        sarr = (C.c_void_p * max(1, ns))(*[ptr(a) for a in out["s"]])
        check(lib().ntg_fld_read(self.fname.encode(), 1 if device is not None else 0, C.c_void_p(el.ctypes.data),
                                 *[ptr(out.get(k)) for k in self.KEYS], sarr if ns else None, ns))
        out["glb_el"] = el
        out.update(h)
        return out


# masked ops: the reference's cuda_* entry points (math_ext.cu:49-108)
def _mi(mask):
    return C.byref(C.c_int(int(mask.numel())))


def _queue():
    lib().ntg_set_glb_queue(_stream())


def cadd_mask(a, c, mask):
    _queue()
    lib().cuda_cadd_mask(_ptr(a), C.byref(C.c_double(c)), C.byref(C.c_int(a.numel())), _ptr(mask, torch.int32),
                         _mi(mask))
    check_last("cuda_cadd_mask")


def invcol1_mask(a, mask):
    _queue()
    lib().cuda_invcol1_mask(_ptr(a), C.byref(C.c_int(a.numel())), _ptr(mask, torch.int32), _mi(mask))
    check_last("cuda_invcol1_mask")


def cmult_mask(a, c, mask):
    _queue()
    lib().cuda_cmult_mask(_ptr(a), C.byref(C.c_double(c)), C.byref(C.c_int(a.numel())), _ptr(mask, torch.int32),
                          _mi(mask))
    check_last("cuda_cmult_mask")


def col2_mask(a, b, mask):
    _queue()
    lib().cuda_col2_mask(_ptr(a), _ptr(b), C.byref(C.c_int(a.numel())), _ptr(mask, torch.int32), _mi(mask))
    check_last("cuda_col2_mask")


def col3_mask(a, b, c, mask):
    _queue()
    lib().cuda_col3_mask(_ptr(a), _ptr(b), _ptr(c), C.byref(C.c_int(a.numel())), _ptr(mask, torch.int32), _mi(mask))
    check_last("cuda_col3_mask")


def sub3_mask(a, b, c, mask):
    _queue()
    lib().cuda_sub3_mask(_ptr(a), _ptr(b), _ptr(c), C.byref(C.c_int(a.numel())), _ptr(mask, torch.int32), _mi(mask))
    check_last("cuda_sub3_mask")


def glsc2_mask(a, b, mask) -> float:
    _queue()
    v = lib().cuda_glsc2_mask(_ptr(a), _ptr(b), C.byref(C.c_int(a.numel())), _ptr(mask, torch.int32), _mi(mask))
    check_last("cuda_glsc2_mask")
    return float(v)

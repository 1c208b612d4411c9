"""GB300-native spectral-element Helmholtz/Poisson hot path.

Python host side over the C ABI (include/ntgb300.h) of ``lib/libntgb300.so``.
The classes mirror the Neko/neko-top interfaces the reference drives on this
path, with the same names and argument meaning:

    coef_t / dofmap      mesh, geometric factors, mult, gs maps   (Neko coef_t, gs_t%init, dofmap_t)
    gs_t.op              direct stiffness summation              (gs_t%op(u, n, GS_OP_ADD))
    ax_helm_t.compute    w = h1 K u + h2 B u                     (ax_helm)
    jacobi_t             update / solve                          (pc_t, jacobi)
    krylov_solver_factory -> ksp.solve / solve_coupled           (ksp_t, ksp_monitor_t)
    projection_t         pre_solving / post_solving              (projection_t)
    RAMP_mapping_t       apply_forward / apply_backward          (sources/mapping_functions/RAMP_mapping.f90)
    PDE_filter_t         apply_forward / apply_backward          (sources/mapping_functions/PDE_filter_mapping.f90)
    simple_brinkman_source_term_t.compute                        (sources/source_terms/simple_brinkman_source_term.f90)
    cadd_mask ... glsc2_mask                                     (sources/neko_ext/math/math_ext.f90)
    opgrad, dudxyz, cdtp, conv1, curl                            (Neko operators, as the adjoint terms call them)
    adv_lin_no_dealias_t.compute_adjoint / compute_linear        (sources/adjoint/adv_adjoint_no_dealias.f90)
    adv_lin_dealias_t.compute_adjoint / compute_linear           (sources/adjoint/adv_adjoint_dealias.f90)
    adjoint_minimum_dissipation_source_term_t.compute            (sources/source_terms/adjoint_minimum_dissipation_source_term.f90)
    pnpn_prs_res_t / pnpn_vel_res_t .compute                     (prs_res / vel_res, sources/adjoint/adjoint_pnpn.f90:716-753)
    pnpn_step_t.step                                             (the pressure + velocity solve sequence, :714-801)
    mma_t.update / KKT                                           (sources/mma/mma.f90, on the GPU)
    fld_file_t.write / read                                      (Nek5000 binary field files, fld_file_output_t)
    nmsh.read / write / coef_from_nmsh / face_mask               (Neko's .nmsh mesh files, the cases' "mesh_file")
    load_case, solver_from_case, build_solver                    (solver wiring from the case file, adjoint_scheme.f90:693-851)

Field arguments are CUDA tensors (torch) laid out like Neko's x(lx,ly,lz,nelv):
contiguous, i fastest.  Only their device pointers cross the boundary.  There
is no CPU fallback: if the CUDA library is missing, importing the native
module raises.
"""
from __future__ import annotations

from ._native import (GS_OP_ADD, GS_OP_MAX, GS_OP_MIN, GS_OP_MUL, KSP_CG, KSP_CG_MIXED, KSP_FCG_MIXED, KSP_GMRES,
                      KSP_GMRES_MIXED, NTG_BREAKDOWN,
                      NTG_MAXITER, NTG_NONFINITE, NTG_OK, NtgError, library_path, lib)
from .api import (PDE_filter_t, RAMP_mapping_t, SolveSequence, adjoint_minimum_dissipation_source_term_t,
                  adv_lin_dealias_t, adv_lin_no_dealias_t, ar1_modes, ax_helm_t, build_box, cadd_mask, cdtp, cmult_mask, coef_t,
                  col2_mask, col3_mask, conv1, curl, dudxyz, fld_file_t, glsc2_mask, glsc3, gs_t, invcol1_mask, jacobi_t, opgrad,
                  build_solver, krylov_solver_factory, ksp_monitor_t, learned_guess_t, load_case, mask_face_xmax, mma_t,
                  permeability, profiler_end_region, profiler_region, profiler_start_region, solver_config_t,
                  solver_from_case,
                  pnpn_prs_res_t,
                  pnpn_step_t, pnpn_vel_res_t, projection_t, schwarz_t,
                  sens_min_dissipation, simple_brinkman_source_term_t, sub3_mask)

from . import dist  # noqa: E402  (element-partitioned solves across ranks)
from . import dofmap  # noqa: E402  (global node ids from element-vertex connectivity)
from . import nmsh  # noqa: E402  (Neko's .nmsh mesh files)

__all__ = [
    "GS_OP_ADD", "GS_OP_MUL", "GS_OP_MIN", "GS_OP_MAX", "KSP_CG", "KSP_CG_MIXED", "KSP_FCG_MIXED", "KSP_GMRES",
    "KSP_GMRES_MIXED", "NTG_OK", "NTG_MAXITER",
    "NTG_BREAKDOWN", "NTG_NONFINITE", "NtgError", "library_path", "lib", "coef_t", "gs_t", "ax_helm_t", "jacobi_t",
    "krylov_solver_factory", "ksp_monitor_t", "projection_t", "RAMP_mapping_t", "PDE_filter_t",
    "simple_brinkman_source_term_t", "cadd_mask", "invcol1_mask", "cmult_mask", "col2_mask", "col3_mask",
    "sub3_mask", "glsc2_mask", "glsc3", "permeability", "sens_min_dissipation", "build_box", "mask_face_xmax",
    "learned_guess_t", "SolveSequence", "profiler_start_region", "profiler_end_region", "profiler_region", "ar1_modes", "schwarz_t", "dist", "dofmap", "nmsh", "opgrad", "dudxyz", "cdtp", "conv1", "curl",
    "adv_lin_no_dealias_t", "adv_lin_dealias_t", "adjoint_minimum_dissipation_source_term_t", "pnpn_prs_res_t", "pnpn_vel_res_t", "pnpn_step_t", "mma_t", "fld_file_t", "load_case", "solver_from_case",
    "solver_config_t", "build_solver",
]

"""Solver wiring from a Neko case file (the reference's lookup in
sources/adjoint/adjoint_scheme.f90:693-851): the tolerant parser and the
adjoint -> fluid key fallback with its defaults.  Host logic only."""
import pytest

CASE = """
{
    "version": 1.0,
    "case": {
        // a comment, and "quotes, }" inside a string stay
        "mesh_file": "box, v2.nmsh",
        "numerics": {"polynomial_order": 7, "dealias": true,},
        "fluid": {
            "velocity_solver": {
                "type": "cg",
                "preconditioner": "jacobi",
                "projection_space_size": 0,
                "absolute_tolerance": 1e-6,
                "max_iterations": 800
            },
            "pressure_solver": {
                "type": "gmres",
                "preconditioner": "hsmg",
                "absolute_tolerance": 1e-4,
            },
        },
        "adjoint": {
            "pressure_solver": {"absolute_tolerance": 1e-7, "max_iterations": 300},
            "velocity_solver": {"projection_hold_steps": 3},
            "projection_hold_steps": 2,
        },
    },
}
"""


def test_parser_keeps_strings_and_drops_comments(pkg):
    p = pkg.load_case(CASE)
    assert p["case"]["mesh_file"] == "box, v2.nmsh"
    assert p["case"]["numerics"] == {"polynomial_order": 7, "dealias": True}


def test_adjoint_keys_fall_back_to_fluid(pkg):
    p = pkg.load_case(CASE)
    prs = pkg.solver_from_case(p, "pressure")
    assert (prs.ksp, prs.pc, prs.abstol, prs.max_iter) == ("gmres", "hsmg", 1e-7, 300)
    # a projection key directly under case.adjoint is not a solver key: the
    # reference reads them only under <field>_solver, so the default 5 holds
    assert prs.projection_space_size == 20 and prs.projection_hold_steps == 5
    vel = pkg.solver_from_case(p, "velocity")
    assert (vel.ksp, vel.pc, vel.abstol, vel.max_iter, vel.projection_space_size) == ("cg", "jacobi", 1e-6, 800, 0)
    assert vel.projection_hold_steps == 3


def test_missing_required_key(pkg):
    with pytest.raises(KeyError):
        pkg.solver_from_case({"case": {"fluid": {"pressure_solver": {"type": "cg"}}}}, "pressure")
    with pytest.raises(ValueError):
        pkg.solver_from_case({}, "temperature")


def test_unbuilt_solver_kinds_are_refused_before_any_gpu_call(pkg):
    cfg = pkg.solver_config_t("pressure", "bicgstab", "jacobi", 1e-6, 800, 0, 5)
    with pytest.raises(ValueError):
        pkg.build_solver(None, cfg)
    cfg = pkg.solver_config_t("pressure", "cg", "sx_jacobi", 1e-6, 800, 0, 5)
    with pytest.raises(ValueError):
        pkg.build_solver(None, cfg)

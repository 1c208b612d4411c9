#!/usr/bin/env python
"""Benchmark: time to a 1e-10 relative residual of the SEM Brinkman
pressure-Poisson sequence on one GB300 with the learned initial guess and
the FP32-inner / FP64-refined CG, against the plain FP64 drop-in
(Jacobi-PCG with Neko's residual projection) on the same GPU, plus the Ax
GDOF/s of both precisions.

Workload (default, --config c5seq): 64^3 hex elements, N = 7 (134M local
DOFs), box deformed by a seeded sinusoid of amplitude 0.05 h per axis,
Brinkman pressure-Poisson h1 = 1, h2 = chi(rho) (RAMP q = 8, chimax = 1e4,
rho = 12 Gaussian blobs moved by a seeded 1% perturbation every 20 solves),
Dirichlet face x = 1, a 200-solve sequence of right-hand sides from 32
Fourier modes with AR(1) amplitudes (rho = 0.98).  The network trains
online on solves 1-100; one step = one solve of the evaluation half (101 on)
with its RHS resident in HBM; `e2e` times further solves through the public
API with the RHS copied from pinned host memory and the solution copied
back.  Inputs are synthetic (seeded generators in the library) and larger
than L2.  --config c1/c2/c3/c5 times single solves from a zero guess.

--impl reference times the reference algorithm's CPU implementation (the C
oracle: FP64 Jacobi-PCG, matrix-free sum factorisation, OpenMP) on the host
cores; each step is a bounded sample of CG iterations, and the value scales
it by the iterations of a full solve (the line says by how many).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "Poisson solve time to 1e-10 & Ax GDOF/s: learned+FP32 vs plain FP64, 1 GB300"

CONFIGS = {
    "c1": dict(E=(8, 8, 8), amp=0.0, case="brinkman_uniform", dirichlet=False,
               desc="8^3 affine unit cube, N=7, h1=1, h2=chi(rho) RAMP q=8 chimax=1e4, rho~U[0,1], "
                    "zero-mean uniform RHS, Jacobi-PCG to 1e-10 rel"),
    "c2": dict(E=(32, 32, 32), amp=0.05, case="poisson_fourier", dirichlet=True,
               desc="32^3 deformed hex (0.05h sinusoid), N=7, pressure-Poisson h1=1 h2=0, Dirichlet x=1, "
                    "16 Fourier modes ~|k|^-2, solve to 1e-10 rel"),
    "c3": dict(E=(32, 32, 32), amp=0.05, case="brinkman_blobs", dirichlet=True,
               desc="32^3 deformed hex, N=7, Brinkman Helmholtz h1=1/Re=0.01, h2=chi(12 Gaussian blobs), "
                    "Dirichlet x=1, 16 Fourier modes, solve to 1e-10 rel"),
    "c2m": dict(E=(24, 24, 24), amp=0.05, case="poisson_fourier", dirichlet=True,
                desc="24^3 deformed hex (0.05h sinusoid), N=7 (7.1M local DOFs), the c2 physics on a mesh sized for "
                     "ncu captures (inputs still above L2)"),
    "c5": dict(E=(64, 64, 64), amp=0.05, case="poisson_fourier", dirichlet=True,
               desc="64^3 deformed hex, N=7 (134M local DOFs), pressure-Poisson, Dirichlet x=1, "
                    "16 Fourier modes, solve to 1e-10 rel"),
}
LX = 8
MESH_SEED, RHS_SEED, RHO_SEED = 1, 2, 3
RTOL = 1e-10


# ---------------------------------------------------------------------------
# helpers shared by both arms
# ---------------------------------------------------------------------------
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def max_over_ranks(value: float, ws: int) -> float:
    """Maximum of a per-rank float (time) over all ranks; identity at 1 rank."""
    if ws == 1:
        return value
    import torch
    import torch.distributed as dist
    dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend() == "nccl" else torch.device("cpu")
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(ws: int):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    _count = 0

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.proc = None
        ClockSampler._count += 1
        self.path = os.path.join(os.environ.get("NTG_CLOCKS_DIR", tempfile.gettempdir()),
                                 f"clocks_{os.getpid()}_{ClockSampler._count}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for nm, v in zip(names, p[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_min_mhz": min(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_traffic(kernel, n, ncoef):
    """DRAM bytes per launch of `kernel` from the committed ncu capture
    (profiles/traffic.json), scaled to n local DOFs; None when the capture
    was taken with a different coefficient set."""
    try:
        tab = json.load(open(os.path.join(ROOT, "profiles", "traffic.json")))
    except Exception:
        return None
    for key, t in tab.items():
        if isinstance(t, dict) and key.split("/")[0] == kernel and t.get("coefficients", 0) == ncoef:
            return int(round(t["bytes_per_launch"] * n / t["n_local_dofs"]))
    return None


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))), "measured"
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def setup_gpu_case(pkg, cfg, dev):
    import torch
    ex, ey, ez = cfg["E"]
    coef = pkg.coef_t.box(ex, ey, ez, LX, amp=cfg["amp"], seed=MESH_SEED, device=dev)
    ncoef = 0
    if cfg["dirichlet"]:
        coef.set_mask(pkg.mask_face_xmax(ex, ey, ez, LX, device=dev), base=1)
    if cfg["case"] == "poisson_fourier":
        coef.set_coefs(h1c=1.0, ifh2=False)
        f = coef.rhs_assemble(coef.field_fourier(16, RHS_SEED))
    elif cfg["case"] == "brinkman_blobs":
        rho = coef.field_blobs(RHO_SEED, 12, 0.1)
        chi = torch.empty_like(rho)
        pkg.RAMP_mapping_t(0.0, 1e4, 8.0, False).apply_forward(chi, 1.0 - rho)
        coef.set_coefs(h1c=0.01, h2=chi, ifh2=True)
        ncoef = 1
        f = coef.rhs_assemble(coef.field_fourier(16, RHS_SEED))
    else:  # brinkman_uniform
        rho = coef.field_uniform(RHO_SEED, 2, 0.0, 1.0)
        chi = torch.empty_like(rho)
        pkg.RAMP_mapping_t(0.0, 1e4, 8.0, False).apply_forward(chi, 1.0 - rho)
        coef.set_coefs(h1c=1.0, h2=chi, ifh2=True)
        ncoef = 1
        b = coef.field_uniform(RHS_SEED, 3, -1.0, 1.0)
        g = coef.geometry()
        b = b - (b * g["mult"]).sum() / coef.nu
        f = b
    torch.cuda.synchronize()
    return coef, f, ncoef


def time_solves(ksp, x, f, k, ev):
    import torch
    mons = []
    e0, e1 = ev(), ev()
    e0.record()
    for _ in range(k):
        x.zero_()
        mons.append(ksp.solve(x, f))
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1e3, mons


def run_kernels_only(args, pkg, coef, f, dev):
    """A few launches of each hot kernel on the workload (for profiler
    captures): FP64 Ax, FP32 Ax, gs, 24 iterations of the mixed solver (with
    the two-level Schwarz when --pc schwarz2), and one forward pass of the
    learned guess's network over all elements (tensor-core GEMMs)."""
    import torch
    n = coef.n
    ax = pkg.ax_helm_t()
    for dt in (torch.float64, torch.float32):
        u = torch.randn(n, dtype=dt, device=dev)
        w = torch.empty_like(u)
        for _ in range(3):
            ax.compute(w, u, coef)
        pkg.gs_t(coef).op(w)
    ksp = pkg.krylov_solver_factory(coef, "cg_mixed", 24, RTOL)
    if args.pc in ("schwarz", "schwarz2"):
        sw = pkg.schwarz_t(coef, coarse=args.pc == "schwarz2")
        sw.set_fdm_path(args.fdm_path)
        ksp.set_schwarz(sw)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    mon = ksp.solve(x, f)
    torch.cuda.synchronize()
    net = pkg.learned_guess_t(coef, history=4, hidden=64, seed=1)
    E = coef.nelv
    Xb = torch.randint(-16000, 16000, (E, net.F), dtype=torch.int16, device=dev)
    net.forward_raw(Xb, E)
    torch.cuda.synchronize()
    return {"kernels_only": True, "n_local_dofs": n, "iters": mon.iter, "status": mon.status}


SEQUENCES = {
    "c5": dict(E=(64, 64, 64), lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), amp=0.05, nsolves=200, ntrain=100,
               desc="64^3 deformed hex (0.05h sinusoid), N=7 (134M local DOFs); Brinkman Poisson h1=1, h2=chi(rho) "
                    "(RAMP q=8, chimax=1e4, rho = 12 Gaussian blobs, moved by a seeded 1% perturbation every 20 "
                    "solves); RHS = 32 Fourier modes with AR(1) amplitudes (rho=0.98); Dirichlet x=1; 200 solves to "
                    "1e-10, online training on 1-100, evaluation on 101-200"),
    "c4": dict(E=(64, 16, 16), lo=(0.0, 0.0, 0.0), hi=(8.0, 2.0, 2.0), amp=0.05, nsolves=400, ntrain=200,
               desc="channel 64x16x16 hex on [0,8]x[0,2]x[0,2] (0.05h sinusoid), N=7 (8.4M local DOFs); Brinkman "
                    "Poisson h1=1, h2=chi(rho) (RAMP q=8, chimax=1e4, rho = 12 Gaussian blobs, moved by a seeded 1% "
                    "perturbation every 20 solves); RHS = 32 Fourier modes with AR(1) amplitudes (rho=0.98); Dirichlet "
                    "x=8; 400 solves to 1e-10, online training on 1-200, evaluation on 201-400"),
}
DESIGN_EVERY = 20  # the design field moves every 20 solves
GUESS_DESC = {
    "learned_only": "the learned network's guess as the initial guess, behind the zero-guess guard",
    "learned": "the learned network's guess as an extra direction of Neko's residual projection, L={L}",
    "projection": "Neko's residual projection, L={L}",
    "zero": "zero initial guess",
}


class SequenceCase:
    """The seeded Brinkman pressure-Poisson sequence on the device: mesh,
    Dirichlet face, AR(1) right-hand sides and the design field of each
    solve (a 1% perturbation every 20 solves)."""

    def __init__(self, pkg, name, dev):
        import torch
        self.pkg, self.cfg, self.dev = pkg, SEQUENCES[name], dev
        ex, ey, ez = self.cfg["E"]
        self.coef = pkg.coef_t.box(ex, ey, ez, LX, lo=self.cfg["lo"], hi=self.cfg["hi"], amp=self.cfg["amp"],
                                   seed=MESH_SEED, device=dev)
        self.coef.set_mask(pkg.mask_face_xmax(ex, ey, ez, LX, device=dev), base=1)
        self.nsol, self.ntrain = self.cfg["nsolves"], self.cfg["ntrain"]
        self.k, self.ph, self.amps = pkg.ar1_modes(RHS_SEED, 32, self.nsol, rho=0.98)
        self.ramp = pkg.RAMP_mapping_t(0.0, 1e4, 8.0, False)
        self.rho0 = self.coef.field_blobs(RHO_SEED, 12, 0.1)
        self.torch = torch

    def chi(self, t):
        """h2 = chi(rho) of the design that solve t sees."""
        rho = self.rho0.clone()
        for q in range(1, t // DESIGN_EVERY + 1):
            d = self.coef.field_fourier(8, 1000 + q)
            rho.add_(0.01 * d / d.abs().max()).clamp_(0.0, 1.0)
        chi = self.torch.empty_like(rho)
        self.ramp.apply_forward(chi, 1.0 - rho)
        return chi

    def set_design(self, t, chi=None):
        self.coef.set_coefs(h1c=1.0, h2=self.chi(t) if chi is None else chi, ifh2=True)

    def rhs(self, t):
        return self.coef.rhs_assemble(self.coef.field_modes(self.k, self.amps[t], self.ph))


def run_headline_sequence(args, ws, rank, local):
    """The headline: the Brinkman pressure-Poisson sequence (C5: 64^3
    deformed hex, N = 7, 134M local DOFs, 200 solves) solved to 1e-10 with
    the learned initial guess inside Neko's residual projection and the
    FP32-inner / FP64-refined CG with the two-level Schwarz preconditioner.
    The network trains online on solves 1-100; solves from 101 on are the
    evaluation half.  W of them are warm-up, the next K are the timed steps
    (one step = one solve, RHS and design already in HBM), the K after that
    are timed end to end through the public API (RHS copied from pinned host
    memory, solution copied back), the rest of the evaluation half runs
    untimed for its iteration statistics.  Beside it, on the same timed
    solves: projection alone, the zero guess, and the plain FP64 drop-in
    (Jacobi-PCG with Neko's projection) on a sample of them."""
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    L = pkg.lib()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    ev = lambda: torch.cuda.Event(enable_timing=True)
    t_setup = time.time()
    case = SequenceCase(pkg, args.config_seq, dev)
    coef, nsol, ntrain = case.coef, case.nsol, case.ntrain
    n = coef.n
    W, K = args.warmup, args.steps
    t0 = ntrain + W
    if t0 + 2 * K > nsol:
        raise SystemExit(f"--warmup {W} --steps {K}: the evaluation half holds {nsol - ntrain} solves "
                         f"(W + 2K at most)")
    pc = "schwarz2" if args.pc in ("auto", "schwarz2") else args.pc
    # 2.2e-4 = 1e-10^(1/3): three FP64 residuals per solve (measured on this
    # sequence, zero guess: 0.498 s at 3e-4 against 0.518 s at 1e-3, 120 iterations
    # either way; 127 iterations at 1e-4)
    delta = args.delta if args.delta is not None else (2.2e-4 if pc == "schwarz2" else 0.1)
    mode = args.guess

    def new_seq(guess, method="cg_mixed", pc_=pc, delta_=delta):
        return pkg.SolveSequence(coef, method, guess, rtol=RTOL, L=args.proj_l, train_steps=args.train_steps,
                                 seed=3, lr=5e-4, pc=pc_, delta=delta_)

    last_change = lambda t: t - t % DESIGN_EVERY
    case.set_design(0)
    seq = new_seq(mode)
    torch.cuda.synchronize()
    t_setup = time.time() - t_setup

    keep = {}  # solutions of the current design window before t0 (seed the FP64 projection) and the timed ones
    its_train, its_eval, used_eval = [], [], []
    t_train = time.time()

    def solve(t, f):
        if t > 0 and t % DESIGN_EVERY == 0:
            case.set_design(t)
            seq.coefficients_changed()
        seq.training = t < ntrain
        x, mon, used, fn = seq.solve(f)
        assert mon.status == pkg.NTG_OK and mon.res_final <= RTOL * fn * (1 + 1e-9), (t, mon)
        return x, mon, used

    # training half and warm-up; the network as it enters the design window
    # of the timed solves is kept for the comparison runs
    net_snap = None
    for t in range(t0):
        if t == last_change(t0) and seq.net is not None:
            net_snap = seq.net.state()
        x, mon, used = solve(t, case.rhs(t))
        (its_train if t < ntrain else its_eval).append(mon.iter)
        if t >= ntrain:
            used_eval.append(used)
        if t >= last_change(t0):
            keep[t] = x.clone()
    torch.cuda.synchronize()
    t_train = time.time() - t_train

    # the K timed solves: RHS and design fields prepared in HBM beforehand
    fs = [case.rhs(t) for t in range(t0, t0 + K)]
    chis = {t: case.chi(t) for t in range(t0, t0 + K) if t % DESIGN_EVERY == 0}
    torch.cuda.synchronize()
    barrier(ws)
    torch.cuda.synchronize()
    mons = []
    l0 = int(L.ntg_launch_count())
    torch.cuda.nvtx.range_push("timed_solves")
    with ClockSampler(local) as clk:
        e0, e1 = ev(), ev()
        e0.record()
        for q, t in enumerate(range(t0, t0 + K)):
            if t % DESIGN_EVERY == 0:
                case.set_design(t, chis[t])
                seq.coefficients_changed()
            seq.training = False
            x, mon, used, fn = seq.solve(fs[q])
            mons.append((mon, fn, used))
            if q < args.fp64_sample:
                keep[t] = x.clone()
        e1.record()
        torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    launches = int(L.ntg_launch_count()) - l0
    barrier(ws)
    t_timed = max_over_ranks(e0.elapsed_time(e1) / 1e3, ws)
    for mon, fn, used in mons:
        assert mon.status == pkg.NTG_OK and mon.res_final <= RTOL * fn * (1 + 1e-9), mon
        its_eval.append(mon.iter)
        used_eval.append(used)
    del fs

    # end to end through the public API: per step, the RHS is copied from
    # pinned host memory and the solution back, inside the timed region
    f_h = torch.empty(n, dtype=torch.float64).pin_memory()
    x_h = torch.empty(n, dtype=torch.float64).pin_memory()
    f_d = torch.empty(n, dtype=torch.float64, device=dev)
    t_e2e = 0.0
    e2e_steps = []
    clk_e2e = ClockSampler(local)
    clk_e2e.__enter__()
    for t in range(t0 + K, t0 + 2 * K):
        f_h.copy_(case.rhs(t))  # prepared untimed
        chi_t = case.chi(t) if t % DESIGN_EVERY == 0 else None
        torch.cuda.synchronize()
        a, b = ev(), ev()
        c1, c2 = ev(), ev()  # inside the step: the end of the H2D copy, the start of the D2H copy
        a.record()
        f_d.copy_(f_h, non_blocking=True)
        c1.record()
        if chi_t is not None:
            case.set_design(t, chi_t)
            seq.coefficients_changed()
        seq.training = False
        x, mon, used, fn = seq.solve(f_d)
        c2.record()
        x_h.copy_(x, non_blocking=True)
        b.record()
        torch.cuda.synchronize()
        t_e2e += a.elapsed_time(b) / 1e3
        e2e_steps.append((round(a.elapsed_time(b), 1), round(a.elapsed_time(c1), 1), round(c2.elapsed_time(b), 1),
                          mon.iter))
        assert mon.status == pkg.NTG_OK, mon
        its_eval.append(mon.iter)
        used_eval.append(used)
    clk_e2e.__exit__(None, None, None)
    t_e2e = max_over_ranks(t_e2e, ws)

    # the rest of the evaluation half, untimed (iteration statistics)
    if not args.short_eval:
        for t in range(t0 + 2 * K, nsol):
            x, mon, used = solve(t, case.rhs(t))
            its_eval.append(mon.iter)
            used_eval.append(used)

    # live per-kernel device times inside one more solve of the sequence
    L.ntg_timer_reset()
    L.ntg_timer_enable(1)
    tprof = min(nsol - 1, t0 + 2 * K)
    seq.training = False
    _, mon_prof, _, _ = seq.solve(case.rhs(tprof))
    torch.cuda.synchronize()
    L.ntg_timer_enable(0)
    ktimes = read_timers(L, mon_prof.iter)
    seq = None
    torch.cuda.empty_cache()

    # comparison modes on the same timed solves (same design window)
    def window_run(guess, method="cg_mixed", pc_=pc, delta_=delta, seed_from=None, nt=K):
        """The same K solves with another guess mode, timed the same way
        (one bracket of CUDA events around all of them, design updates
        included).  Projection modes replay the design window from its
        start; a learned mode starts from the trained network as it was at
        the window's start."""
        case.set_design(last_change(t0))
        s2 = new_seq(guess, method, pc_, delta_)
        s2.training = False
        if s2.net is not None:
            s2.net.load_state(net_snap)
        start = last_change(t0)
        if guess == "zero" or method == "cg":
            start = t0
        if seed_from is not None:
            for t in range(last_change(t0), t0):
                s2.record(case.rhs(t), seed_from[t])
        for t in range(start, t0):
            s2.solve(case.rhs(t))
        fs2 = [case.rhs(t) for t in range(t0, t0 + nt)]
        chis2 = {t: case.chi(t) for t in range(t0, t0 + nt) if t % DESIGN_EVERY == 0}
        torch.cuda.synchronize()
        mons2, xs = [], []
        a, b = ev(), ev()
        a.record()
        for q, t in enumerate(range(t0, t0 + nt)):
            if t % DESIGN_EVERY == 0:
                case.set_design(t, chis2[t])
                s2.coefficients_changed()
            x, mon, used, fn = s2.solve(fs2[q])
            mons2.append((mon, fn))
            if method == "cg":
                xs.append(x.clone())
        b.record()
        torch.cuda.synchronize()
        for mon, fn in mons2:
            assert mon.status == pkg.NTG_OK and mon.res_final <= RTOL * fn * (1 + 1e-9), (guess, mon)
        del s2, fs2
        torch.cuda.empty_cache()
        return [m.iter for m, _ in mons2], a.elapsed_time(b) / 1e3 / nt, xs

    extra = {}
    t_ours = t_timed / K
    if not args.no_compare:
        for g in ("learned_only", "learned", "projection", "zero"):
            if g == mode or (g.startswith("learned") and net_snap is None):
                continue
            its, sec, _ = window_run(g)
            extra[g] = {"iters_mean": round(statistics.mean(its), 2), "s_per_solve": round(sec, 5)}
    # the plain FP64 drop-in (Jacobi-PCG + Neko's projection, L = 20) on the
    # first solves of the timed window, its basis seeded with this design
    # window's earlier solutions
    fp64 = None
    if args.fp64_sample > 0:
        its, t64, xs = window_run("projection", "cg", "jacobi", None, seed_from=keep, nt=args.fp64_sample)
        errs = [float(torch.linalg.norm(keep[t0 + q] - xs[q]) / torch.linalg.norm(xs[q])) for q in range(len(xs))]
        ours_same = statistics.mean(float(m[0].iter) for m in mons[:len(xs)])
        fp64 = {"method": "FP64 Jacobi-PCG + residual projection (L=%d), the plain drop-in" % args.proj_l,
                "s_per_solve": round(t64, 4), "iters_mean": round(statistics.mean(its), 1), "solves": len(xs),
                "error_vs_fp64_solution": max(errs), "ours_iters_same_solves": ours_same}
    del keep
    torch.cuda.empty_cache()

    # Ax alone at this size: both precisions, cold L2 per launch (a 256 MB
    # write between launches), against the in-solve FP32 launches
    ax = ax_rates(pkg, coef, dev)
    pk, pk_kind = peaks()
    ncoef = 1  # h2 = chi * B precombined
    ax32 = ktimes.get("ax_fp32")
    bpd = (2 + 6 + ncoef) * 4
    t_in = ax32["avg_us"] * 1e-6 if ax32 else ax["fp32_s"]
    roof = {"kernel": "k_ax_helm_f32_tma (FP32 Ax inside the timed solves)", "bound": "hbm",
            "achieved": round(bpd * n / t_in / 1e9, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": round(bpd * n / t_in / 1e9 / pk["hbm_gbs"], 4), "peak_source": pk_kind,
            "bytes_per_dof": bpd, "standalone_cold": {
                "us": round(ax["fp32_s"] * 1e6, 1), "achieved": round(bpd * n / ax["fp32_s"] / 1e9, 1),
                "frac": round(bpd * n / ax["fp32_s"] / 1e9 / pk["hbm_gbs"], 4)},
            "traffic": args.traffic if args.traffic is not None else measured_traffic("k_ax_helm_f32_tma", n, ncoef)}
    fdm = ktimes.get("schwarz_fdm")
    roof_fdm = None
    if fdm:
        # algorithmic bytes per element: the extended box's values of r are
        # read once per element in the ideal (each local DOF once, 4 B) and
        # the extended result written (LE^3 x 4 B, LE = lx + 2), plus the
        # element's six scalars
        E = coef.nelv
        b_fdm = 4 * n + 4 * E * (LX + 2) ** 3 + 6 * 4 * E
        roof_fdm = {"kernel": "k_fdm<8> (Schwarz local solves, the largest share of a solve)", "bound": "hbm",
                    "achieved": round(b_fdm / (fdm["avg_us"] * 1e-6) / 1e9, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
                    "frac": round(b_fdm / (fdm["avg_us"] * 1e-6) / 1e9 / pk["hbm_gbs"], 4), "peak_source": pk_kind,
                    "bytes_per_launch": b_fdm, "avg_us": fdm["avg_us"],
                    "traffic": measured_traffic("k_fdm", n, 0),
                    "algorithmic_note": "4 B per local DOF of r read + (lx+2)^3 x 4 B per element of extended results "
                                        "written + 6 scalars per element"}
    ax64 = ktimes.get("ax_fp64")
    t_k64 = ax64["avg_us"] * 1e-6 if ax64 else ax["fp64_s"]
    roof64 = {"kernel": "k_ax_helm<double,8> (FP64 Ax: residual replacements, projection)", "bound": "fp64",
              "achieved": round(116.0 * n / t_k64 / 1e9, 1), "peak": FP64_TFLOPS * 1e3, "unit": "GFLOP/s",
              "frac": round(116.0 * n / t_k64 / 1e9 / (FP64_TFLOPS * 1e3), 4),
              "peak_source": "FP64 FMA-chain probe, bench.py --fp64-peak"}

    ev_its = its_eval
    out = {
        "metric": METRIC,
        "value": round(ws * K / t_timed, 4),
        "unit": "solves/s",
        "n_gpus": ws,
        "steps": K,
        "warmup": W,
        "ms_per_step": round(t_timed / K * 1e3, 3),
        "s_per_solve": round(t_timed / K, 5),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 inner / f64 outer (bf16 network)",
        "data": "synthetic (seeded generators; no dataset)",
        "config": {"workload": f"{args.config_seq} sequence: {case.cfg['desc']}", "n_local_dofs": n,
                   "n_unique_dofs": coef.nu,
                   "method": f"guess '{mode}' ({GUESS_DESC[mode].format(L=args.proj_l)}) + "
                             f"cg_mixed (FP32 PCG, {pc} preconditioner, FP64 reliable updates at delta={delta:g})",
                   "step": f"one solve of the evaluation half to 1e-10 (solves {t0 + 1}-{t0 + K} of {nsol}; "
                           f"{ntrain} training solves and {W} warm-up solves before)",
                   "l2": "inputs larger than L2 (FP32 G 3.2 GB, FP64 G 6.4 GB at 64^3)",
                   "parallelism": "replicas only" if ws > 1 else "1 GPU"},
        "iterations": {"timed_mean": round(statistics.mean(m[0].iter for m in mons), 2),
                       "eval_mean": round(statistics.mean(ev_its), 2), "eval_solves": len(ev_its),
                       "train_mean": round(statistics.mean(its_train), 2),
                       "fp64_ax_per_solve": round(statistics.mean(m[0].fp64_ax for m in mons), 2),
                       "guess_used": {u: used_eval.count(u) for u in sorted(set(used_eval))}},
        "compare_same_solves": extra,
        "fp64_dropin": fp64,
        "speedup_vs_fp64_dropin": round(fp64["s_per_solve"] / t_ours, 2) if fp64 else None,
        "ax_gdof_s": {"fp64": round(n / ax["fp64_s"] / 1e9, 3), "fp32": round(n / ax["fp32_s"] / 1e9, 3),
                      "fp32_in_solve": round(n / t_in / 1e9, 3)},
        "roofline": roof,
        "roofline_fdm": roof_fdm,
        "roofline_fp64_ax": roof64,
        "kernels_in_one_solve": ktimes,
        "e2e": {"value": round(ws * K / t_e2e, 4), "unit": "solves/s", "h2d_bytes_per_step": int(n * 8),
                "d2h_bytes_per_step": int(n * 8),
                "note": "each step timed alone (CUDA events): H2D copy of its RHS from pinned memory, the solve "
                        "through SolveSequence.solve, D2H copy of x; the RHS is prepared untimed between steps",
                "steps_ms_h2d_d2h_iters": e2e_steps, "timed_iters": [m.iter for m, _, _ in mons],
                "clocks": clk_e2e.summary()},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "setup_s": round(t_setup, 3),
        "train_s": round(t_train, 2),
    }
    if rank == 0 and ws == 1 and not args.no_cpu:
        out["cpu_baseline"] = cpu_sample_seq(args.config_seq, args.cpu_iters, fp64["iters_mean"] if fp64 else None)
    return out


def read_timers(L, iters=None):
    """Per-kernel device times of the solve(s) timed with the library's
    timers.  The host polls the device stop flag every 16 iterations, so up
    to 15 launches of each per-iteration FP32 kernel run after convergence
    and return at once; with `iters` (the iterations done) their average is
    taken over the iterations that did work."""
    import ctypes as C
    names = {0: "ax_fp64", 1: "ax_fp32", 2: "gs_fp64", 3: "gs_fp32", 4: "cg_update_fp64", 5: "cg_update_fp32",
             6: "cg_dir_fp64", 7: "cg_dir_fp32", 8: "precond_fp32", 9: "schwarz_fdm", 10: "schwarz_coarse",
             11: "schwarz_pull"}
    per_iter = {"ax_fp32", "gs_fp32", "cg_update_fp32", "cg_dir_fp32", "precond_fp32", "schwarz_fdm",
                "schwarz_coarse", "schwarz_pull"}
    out = {}
    for i, nm in names.items():
        ms, cnt = C.c_double(), C.c_longlong()
        L.ntg_timer_read(i, C.byref(ms), C.byref(cnt))
        if cnt.value:
            eff = min(cnt.value, iters) if (iters and nm in per_iter) else cnt.value
            out[nm] = {"total_ms": round(ms.value, 4), "launches": cnt.value, "launches_working": eff,
                       "avg_us": round(ms.value / eff * 1e3, 2)}
    # shares of the solve: the preconditioner's parts are inside precond_fp32
    tot = sum(v["total_ms"] for k, v in out.items() if not k.startswith("schwarz_")) or 1.0
    for v in out.values():
        v["share"] = round(v["total_ms"] / tot, 4)
    return out


def ax_rates(pkg, coef, dev, reps=10):
    """Seconds per Ax launch, FP64 and FP32, each launch timed alone with
    CUDA events after a 256 MB write that evicts L2."""
    import torch
    n = coef.n
    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev)
    ax = pkg.ax_helm_t()
    res = {}
    for dt, key in ((torch.float64, "fp64_s"), (torch.float32, "fp32_s")):
        u = torch.randn(n, dtype=dt, device=dev)
        w = torch.empty_like(u)
        for _ in range(3):
            ax.compute(w, u, coef)
        tt = []
        for _ in range(reps):
            flush.fill_(1.0)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            ax.compute(w, u, coef)
            b.record()
            torch.cuda.synchronize()
            tt.append(a.elapsed_time(b) / 1e3)
        res[key] = statistics.median(tt)
        del u, w
    return res


def run_sequence(args, local):
    """A right-hand-side sequence solved with each initial-guess mode (zero,
    projection, projection + learned direction, learned guess alone), the
    network trained online on the first half and frozen on the second; the
    plain FP64 drop-in (Jacobi-PCG, zero guess and projection) on a sample
    of the evaluation half."""
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    cfg = SEQUENCES[args.sequence]
    ex, ey, ez = cfg["E"]
    coef = pkg.coef_t.box(ex, ey, ez, LX, lo=cfg["lo"], hi=cfg["hi"], amp=cfg["amp"], seed=MESH_SEED, device=dev)
    coef.set_mask(pkg.mask_face_xmax(ex, ey, ez, LX, device=dev), base=1)
    nsol, ntrain = cfg["nsolves"], cfg["ntrain"]
    k, ph, amps = pkg.ar1_modes(RHS_SEED, 32, nsol, rho=0.98)
    ramp = pkg.RAMP_mapping_t(0.0, 1e4, 8.0, False)
    rho0 = coef.field_blobs(RHO_SEED, 12, 0.1)

    def design(t):  # the design field of solve t: a 1% perturbation every 20 solves
        rho = rho0.clone()
        for q in range(1, t // 20 + 1):
            d = coef.field_fourier(8, 1000 + q)
            rho.add_(0.01 * d / d.abs().max()).clamp_(0.0, 1.0)
        chi = torch.empty_like(rho)
        ramp.apply_forward(chi, 1.0 - rho)
        return chi

    ev = lambda: torch.cuda.Event(enable_timing=True)
    pc = "schwarz2" if args.pc in ("auto", "schwarz2") else args.pc
    delta = args.delta if args.delta is not None else (2.2e-4 if pc == "schwarz2" else 0.1)
    modes = tuple(args.seq_modes.split(","))
    res = {}
    for mode in modes:
        coef.set_coefs(h1c=1.0, h2=design(0), ifh2=True)
        seq = pkg.SolveSequence(coef, "cg_mixed", mode, rtol=RTOL, L=args.proj_l, train_steps=30, seed=3, lr=5e-4,
                                pc=pc, delta=delta)
        if seq.sw is not None and args.mass_term:
            seq.sw.set_mass_term(True)
        its, secs = [], []
        for t in range(nsol):
            if t > 0 and t % 20 == 0:
                coef.set_coefs(h1c=1.0, h2=design(t), ifh2=True)
                seq.coefficients_changed()
            seq.training = t < ntrain
            f = coef.rhs_assemble(coef.field_modes(k, amps[t], ph))
            torch.cuda.synchronize()
            e0, e1 = ev(), ev()
            e0.record()
            x, mon, used, fn = seq.solve(f)
            e1.record()
            torch.cuda.synchronize()
            assert mon.status == pkg.NTG_OK and mon.res_final <= RTOL * fn * (1 + 1e-9), (mode, t, mon)
            if t >= ntrain:
                its.append(mon.iter)
                secs.append(e0.elapsed_time(e1) / 1e3)
        res[mode] = {"iters_mean": round(statistics.mean(its), 2), "s_per_solve": round(statistics.mean(secs), 5)}
        del seq
    # the plain FP64 drop-in on a sample of the evaluation half
    sample = list(range(ntrain, min(nsol, ntrain + args.fp64_sample)))  # consecutive, after 8 warm-up solves
    for mode in ("zero", "projection"):
        coef.set_coefs(h1c=1.0, h2=design(0), ifh2=True)
        seq = pkg.SolveSequence(coef, "cg", mode, rtol=RTOL, L=args.proj_l, pc="jacobi")
        its, secs = [], []
        last = 0
        for t in sorted(set(list(range(max(0, sample[0] - args.fp64_warm), sample[0])) + sample)):
            if t // 20 != last // 20:
                coef.set_coefs(h1c=1.0, h2=design(t), ifh2=True)
                seq.coefficients_changed()
            last = t
            f = coef.rhs_assemble(coef.field_modes(k, amps[t], ph))
            torch.cuda.synchronize()
            e0, e1 = ev(), ev()
            e0.record()
            x, mon, used, fn = seq.solve(f)
            e1.record()
            torch.cuda.synchronize()
            assert mon.status == pkg.NTG_OK, (mode, t, mon)
            if t in sample:
                its.append(mon.iter)
                secs.append(e0.elapsed_time(e1) / 1e3)
        res["fp64_" + mode] = {"iters_mean": round(statistics.mean(its), 2),
                               "s_per_solve": round(statistics.mean(secs), 5), "solves": len(its)}
        del seq
    best = min(modes, key=lambda m: res[m]["s_per_solve"])
    return {
        "metric": "Brinkman Poisson sequence: time per solve to 1e-10 (evaluation half)", "value":
        res[best]["s_per_solve"], "unit": "s/solve", "higher_is_better": False, "best_mode": best,
        "modes": res, "speedup_vs_fp64_projection": round(res["fp64_projection"]["s_per_solve"] /
                                                          res[best]["s_per_solve"], 2),
        "config": {"workload": cfg["desc"], "method": f"cg_mixed with {pc}, FP64 replacements at delta={delta:g}",
                   "n_local_dofs": coef.n}, "n_gpus": 1, "data": "synthetic (seeded generators; no dataset)",
    }


FP64_TFLOPS = 1.2556  # FP64 FMA roof measured by `bench.py --fp64-peak` (the probe library libntgb300_probe.so) on GB300


def run_terms(args, local):
    """The FP64 terms either side of each solve of the adjoint/forward step,
    each timed alone with CUDA events on the launching stream: the Pn/Pn
    velocity and pressure residuals, the adjoint and linearised advection
    (no dealiasing), the minimum-dissipation forcing, and the FP64 Ax for
    scale.  Fields are seeded random, mu = 0.01, rho = 1, bd = 11/6,
    dt = 1e-3; inputs are larger than L2."""
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    cfg = CONFIGS[args.config]
    coef, _, _ = setup_gpu_case(pkg, cfg, dev)
    coef.metrics()
    n = coef.n
    gen = torch.Generator(device=dev).manual_seed(11)
    F = lambda: torch.randn(n, dtype=torch.float64, device=dev, generator=gen)
    u, v, w, ue, ve, we, p, fx, fy, fz = (F() for _ in range(10))
    r = [torch.zeros(n, dtype=torch.float64, device=dev) for _ in range(3)]
    pres = torch.zeros(n, dtype=torch.float64, device=dev)
    ex, ey, ez = cfg["E"]
    face = pkg.mask_face_xmax(ex, ey, ez, LX, device=dev)
    s = torch.zeros(3, face.numel(), dtype=torch.float64, device=dev)
    s[0] = 1.0 / (ey * ez * (LX - 1) ** 2)
    vel, prs = pkg.pnpn_vel_res_t(), pkg.pnpn_prs_res_t()
    adv = pkg.adv_lin_no_dealias_t(coef)
    adv_d = pkg.adv_lin_dealias_t(coef)
    md = pkg.adjoint_minimum_dissipation_source_term_t(r, u, v, w, coef, obj_scale=0.5)
    ax = pkg.ax_helm_t()
    bd, dt = 11.0 / 6.0, 1e-3
    terms = {
        "vel_res": lambda: vel.compute(u, v, w, *r, p, fx, fy, fz, coef, mu=0.01, rho=1.0, bd=bd, dt=dt),
        "prs_res": lambda: prs.compute(p, pres, u, v, w, ue, ve, we, fx, fy, fz, coef, (face, s), None, bd=bd,
                                       dt=dt, mu=0.01, rho=1.0),
        "adjoint_advection": lambda: adv.compute_adjoint(u, v, w, ue, ve, we, *r),
        "linear_advection": lambda: adv.compute_linear(u, v, w, ue, ve, we, *r),
        "adjoint_advection_dealias": lambda: adv_d.compute_adjoint(u, v, w, ue, ve, we, *r),
        "linear_advection_dealias": lambda: adv_d.compute_linear(u, v, w, ue, ve, we, *r),
        "min_dissipation": lambda: md.compute(),
        "ax_helm_fp64": lambda: ax.compute(pres, p, coef),
    }
    # algorithmic FP64 flops per local DOF (lx = 8, lxd = 12; an FMA counts 2):
    # vel_res: 3 x (Helmholtz 117 + mass 3) + pressure gradient 48 + 3 x 8.
    # Dealiased, per element: 9 tensor interpolations (6 to GL, 3 back) of
    # 29,184 FMA each; per GL point the adjoint term's 3 GL gradients (108 FMA),
    # mixing (36 + 9) and per component a D^T of u_i V (36 FMA + 36 products);
    # the linear term's 6 GL gradients (216 FMA) and fluxes (36); / 512 GLL points.
    # Without dealiasing, per node (lx = 8): adjoint 3 gradients (72 FMA),
    # opgrad mixing (36), fluxes V (9), u_i V (9 products) and three D^T (72);
    # linear 6 gradients (144) and mixing (72).
    gl = 12 ** 3
    interp = 12 * 512 + 144 * 64 + 1728 * 8
    flops = {"vel_res": 3 * 120 + 48 + 24, "ax_helm_fp64": 116,
             "adjoint_advection": 2 * (72 + 36 + 9 + 72) + 9, "linear_advection": 2 * (144 + 72),
             "adjoint_advection_dealias": (2 * (9 * interp + gl * (108 + 45 + 3 * 36)) + gl * (6 + 3 * 36)) / 512,
             "linear_advection_dealias": 2 * (9 * interp + gl * (216 + 36)) / 512}
    L = pkg.lib()
    out = {}
    sampler = ClockSampler(local)
    with sampler:
        for name, fn in terms.items():
            for _ in range(args.warmup):
                fn()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            l0 = int(L.ntg_launch_count())
            e0.record()
            for _ in range(args.steps):
                fn()
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / args.steps
            rec = {"ms": round(ms, 4), "gdof_s": round(n / ms / 1e6, 2),
                   "launches": (int(L.ntg_launch_count()) - l0) // args.steps}
            if name in flops:
                tf = flops[name] * n / (ms * 1e-3) / 1e12
                rec["fp64_tflops"] = round(tf, 3)
                rec["frac_of_fp64_roof"] = round(tf / FP64_TFLOPS, 3)
            out[name] = rec
    cpu_threads = None
    if not args.no_cpu:
        cpu, cpu_threads = terms_cpu_baseline(n)
        for name, ms_cpu in cpu.items():
            out[name]["cpu_ms"] = round(ms_cpu, 1)
            out[name]["cpu_over_gpu"] = round(ms_cpu / out[name]["ms"], 1)
    return {"mode": "terms", "config": {"workload": args.config, "desc": cfg["desc"], "n_local_dofs": n,
                                         "l2": "inputs larger than L2"},
            "dtype": "f64", "steps": args.steps, "warmup": args.warmup, "terms": out,
            "cpu_baseline": {"kind": "port", "cores": cpu_threads, "unit": "ms per application",
                             "sample": "the compiled OpenMP restatement (oracle/terms_oracle.c via oracle/terms_c.py, "
                                       "checked against the numpy restatements) on a 6x6x6, lx = 8 box "
                                       "(110,592 DOFs), two timed applications each after one untimed, "
                                       "scaled per DOF to the workload"},
            "clocks": sampler.summary()}


def terms_cpu_baseline(n):
    """Per-application time of each term in the compiled OpenMP restatement
    (oracle/terms_oracle.c, all host threads) on a bounded sample (6^3
    elements, lx = 8), scaled to n local DOFs."""
    import numpy as np
    from oracle import dealias_ref, oracle as orc
    from oracle.terms_c import Terms
    m = orc.build_mesh(6, 6, 6, LX, amp=0.05, seed=MESH_SEED)
    t = Terms(m)
    gl = dealias_ref.GL(m)
    rng = np.random.default_rng(0)
    F = lambda: rng.standard_normal(m.n)
    u, ue, f = [F() for _ in range(3)], [F() for _ in range(3)], [F() for _ in range(3)]
    p = F()
    face = np.nonzero(np.isclose(m.x, m.x.max()))[0]
    surf = (face, np.stack([np.full(face.size, 1e-3), np.zeros(face.size), np.zeros(face.size)]))
    fns = {
        "vel_res": lambda: t.vel_res(u, p, f, 0.01, 1.0, 11 / 6, 1e-3),
        "prs_res": lambda: t.prs_res(p, u, ue, f, 0.01, 1.0, 11 / 6, 1e-3, surf, None),
        "adjoint_advection": lambda: t.advection(f, u, ue, "adjoint"),
        "linear_advection": lambda: t.advection(f, u, ue, "linear"),
        "adjoint_advection_dealias": lambda: t.advection(f, u, ue, "adjoint", gl),
        "linear_advection_dealias": lambda: t.advection(f, u, ue, "linear", gl),
        "min_dissipation": lambda: t.min_dissipation(f, u, 0.5),
        "ax_helm_fp64": lambda: orc.ax_helm(m, p),
    }
    out = {}
    for name, fn in fns.items():
        fn()
        t0 = time.perf_counter()
        for _ in range(2):
            fn()
        out[name] = (time.perf_counter() - t0) / 2 * 1e3 * n / m.n
    return out, orc.num_threads()


def run_mma(args, local):
    """MMA design updates (the optimiser of the topology-optimisation loop)
    with one design variable per local DOF of the workload's mesh: a
    compliance-like objective sum_j w_j / x_j / n (w seeded in [0.5, 2]) and
    the volume constraint mean(x) <= 0.4, x in [1e-3, 1], m = 1.  W untimed
    updates, then K timed (CUDA events, stream synchronised by every
    update); the oracle's numpy restatement timed on a bounded sample."""
    import numpy as np
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    cfg = CONFIGS[args.config]
    ex, ey, ez = cfg["E"]
    n = ex * ey * ez * LX ** 3
    gen = torch.Generator(device=dev).manual_seed(7)
    w = 0.5 + 1.5 * torch.rand(n, dtype=torch.float64, device=dev, generator=gen)
    x = torch.full((n,), 0.5, dtype=torch.float64, device=dev)
    opt = pkg.mma_t(x, n, 1, 1.0, 0.0, 1000.0, 1.0, 1e-3, 1.0)
    dfdx = torch.full((n,), 1.0 / n, dtype=torch.float64, device=dev)

    def step(it):
        df0 = -w / (x * x) / n
        opt.update(it, x, df0, [float(x.mean()) - 0.4], dfdx)

    it = 0
    for _ in range(args.warmup):
        it += 1
        step(it)
    c0 = opt.counts
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        it += 1
        step(it)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / args.steps
    c1 = opt.counts
    newton, trials, levels = ((c1[q] - c0[q]) / args.steps for q in range(3))
    # algorithmic doubles per variable (m = 1): Newton assembly 13, directions
    # 17, each line-search trial 17, each epsilon level's first residual 11,
    # the subproblem generation 20; plus the sensitivity and mean (3)
    dbl = 13 * newton + 17 * newton + 17 * trials + 11 * levels + 20 + 3
    gbs = dbl * 8 * n / (ms * 1e-3) / 1e9
    pk, kind = peaks()
    cpu = None
    if not args.no_cpu:
        # the compiled OpenMP restatement (checked against the numpy one) on a
        # bounded sample of the same problem, all host threads
        from oracle import oracle as orc
        from oracle.mma_c import MMAC
        ns = 2_000_000
        rng = np.random.default_rng(7)
        wc = rng.uniform(0.5, 2.0, ns)
        xc = np.full(ns, 0.5)
        ref = MMAC(xc, 1, 1.0, 0.0, 1000.0, 1.0, 1e-3, 1.0)
        dfc = np.full((1, ns), 1.0 / ns)
        t_cpu = 0.0
        for k in range(1, 4 + 1):
            df0c, fc = -wc / xc ** 2 / ns, np.array([xc.mean() - 0.4])
            t0 = time.perf_counter()
            xc = ref.update(k, xc, df0c, fc, dfc)
            if k > 2:  # the same iterations the GPU leg times come after its warm-up
                t_cpu += time.perf_counter() - t0
        cpu_s = t_cpu / 2 * n / ns
        cpu = {"value": round(cpu_s * 1e3, 1), "unit": "ms", "cores": orc.num_threads(), "kind": "port",
               "sample": f"oracle/mma_oracle.c (OpenMP), updates 3-4 at n = {ns}, scaled to n = {n}"}
    return {"mode": "mma", "metric": "MMA design update time", "unit": "ms", "value": round(ms, 3),
            "higher_is_better": False, "dtype": "f64", "steps": args.steps, "warmup": args.warmup,
            "config": {"workload": f"{args.config} mesh, one design variable per local DOF", "n": n, "m": 1,
                       "l2": "inputs larger than L2"},
            "per_update": {"newton_steps": newton, "line_search_trials": trials, "epsilon_levels": levels,
                           "ms_per_newton_step": round(ms / max(newton, 1), 4)},
            "roofline": {"bound": "fp64", "hbm_achieved": round(gbs, 1), "hbm_peak": pk["hbm_gbs"], "unit": "GB/s",
                         "hbm_frac": round(gbs / pk["hbm_gbs"], 3), "peak_kind": kind,
                         "note": "the kernels are FP64-pipe bound (divisions), see the MMA profile; the HBM figure "
                                 "counts the algorithmic doubles per variable of the whole update, host syncs included"},
            "cpu_baseline": cpu}


def run_ours(args, ws, rank, local):
    import torch
    import __graft_entry__ as ge
    pkg = ge.load_package()
    L = pkg.lib()
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    cfg = CONFIGS[args.config]
    ev = lambda: torch.cuda.Event(enable_timing=True)
    t_setup = time.time()
    coef, f, ncoef = setup_gpu_case(pkg, cfg, dev)
    if args.kernels_only:
        return run_kernels_only(args, pkg, coef, f, dev)
    n = coef.n
    pc = args.pc
    if pc == "auto":  # two-level Schwarz for the pressure-Poisson cases, Jacobi under Brinkman penalisation
        pc = "schwarz2" if cfg["case"] == "poisson_fourier" else "jacobi"
    args.pc_used = pc
    if args.delta is None:
        # reliable-update spacing: the FP32 recurrence drifts with the iterations
        # between FP64 replacements, so a preconditioner that needs few
        # iterations per decade (two-level Schwarz) affords wide spacing;
        # 2.2e-4 = 1e-10^(1/3) makes the 1e-10 solve three FP64 residuals
        # (measured at c2: 0.0563 s against 0.0588 s at 1e-3, same iterations)
        args.delta = 2.2e-4 if pc == "schwarz2" else 0.1
    sw = None
    if args.method == "cg_mixed":
        ksp_mx = pkg.krylov_solver_factory(coef, "cg_mixed", 50000, RTOL)
        ksp_mx.set_inner(args.delta, 1)
        if pc in ("schwarz", "schwarz2"):
            sw = pkg.schwarz_t(coef, coarse=pc == "schwarz2")
            if args.mass_term:
                sw.set_mass_term(True)
            ksp_mx.set_schwarz(sw)
    else:
        ksp_mx = pkg.krylov_solver_factory(coef, "fcg_mixed", 200, RTOL)
        ksp_mx.set_inner(args.inner_rtol, args.inner_max)
    ksp64 = pkg.krylov_solver_factory(coef, "cg", 20000, RTOL)
    x = torch.zeros(n, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    t_setup = time.time() - t_setup

    # warm-up, then the timed steps (inputs > L2: FP32 G alone is 24 B/DOF)
    for _ in range(args.warmup):
        x.zero_()
        ksp_mx.solve(x, f)
    torch.cuda.synchronize()
    barrier(ws)
    torch.cuda.synchronize()
    l0 = int(L.ntg_launch_count())
    torch.cuda.nvtx.range_push("timed_solves")  # lets ncu restrict a launch list to the timed region
    with ClockSampler(dev.index if dev.index is not None else 0) as clk:
        t_mx, mons = time_solves(ksp_mx, x, f, args.steps, ev)
    torch.cuda.nvtx.range_pop()
    launches = int(L.ntg_launch_count()) - l0
    barrier(ws)
    t_mx = max_over_ranks(t_mx, ws)
    x_mx = x.clone()
    for m in mons:
        assert m.status == pkg.NTG_OK and m.res_final <= RTOL * m.rhs_norm * (1 + 1e-9), m

    # the plain FP64 drop-in on the same GPU
    x.zero_()
    ksp64.solve(x, f)  # warm-up
    t64, mons64 = time_solves(ksp64, x, f, args.fp64_steps, ev)
    x64 = x.clone()
    err_vs_fp64 = float(torch.linalg.norm(x_mx - x64) / torch.linalg.norm(x64))

    # Ax alone, both precisions
    def time_ax(dtype, reps=20):
        u = torch.randn(n, dtype=dtype, device=dev)
        w = torch.empty_like(u)
        ax = pkg.ax_helm_t()
        for _ in range(3):
            ax.compute(w, u, coef)
        a, b = ev(), ev()
        a.record()
        for _ in range(reps):
            ax.compute(w, u, coef)
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / 1e3 / reps
    t_ax64, t_ax32 = time_ax(torch.float64), time_ax(torch.float32)

    # live per-kernel device times inside one profiled solve
    L.ntg_timer_reset()
    L.ntg_timer_enable(1)
    x.zero_()
    mon_prof = ksp_mx.solve(x, f)
    torch.cuda.synchronize()
    L.ntg_timer_enable(0)
    ktimes = read_timers(L, mon_prof.iter)

    # roofline of the dominant kernel (FP32 Ax, HBM bound):
    # algorithmic bytes per local DOF = (u in + w out + 6 G + ncoef) * 4 B
    pk, pk_kind = peaks()
    ax32 = ktimes.get("ax_fp32")
    bytes_per_dof = (2 + 6 + ncoef) * 4
    t_launch = ax32["avg_us"] * 1e-6 if ax32 else t_ax32
    achieved = bytes_per_dof * n / t_launch / 1e9
    roof = {"kernel": "k_ax_helm<float,8> (FP32 Ax inside the timed solve)", "bound": "hbm",
            "achieved": round(achieved, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": round(achieved / pk["hbm_gbs"], 4), "peak_source": pk_kind,
            "bytes_per_dof": bytes_per_dof, "traffic": args.traffic if args.traffic is not None
            else measured_traffic("k_ax_helm_f32_tma", n, ncoef)}

    # the FP64 operator against the FP64 compute roof: 116 flop per local DOF
    # (six contractions of 2(N+1) flop each, plus the metric mix), the peak
    # from an FMA-chain probe on GB300 (not in MEASURED_PEAKS.json)
    ax64 = ktimes.get("ax_fp64")
    t_k64 = ax64["avg_us"] * 1e-6 if ax64 else t_ax64  # one FP64 Ax launch
    fp64_peak = FP64_TFLOPS * 1e3
    roof64 = {"kernel": "k_ax_helm<double,8> (FP64 Ax, residual replacements)", "bound": "fp64",
              "achieved": round(116.0 * n / t_k64 / 1e9, 1), "peak": fp64_peak, "unit": "GFLOP/s",
              "frac": round(116.0 * n / t_k64 / 1e9 / fp64_peak, 4), "peak_source": "FP64 FMA-chain probe, bench.py --fp64-peak"}

    # end to end through the public API: host RHS in, host solution out
    f_h = f.cpu().pin_memory()
    x_h = torch.empty(n, dtype=torch.float64).pin_memory()
    f_d = torch.empty_like(f)
    e0, e1 = ev(), ev()
    barrier(ws)
    torch.cuda.synchronize()
    w0 = time.time()
    e0.record()
    for _ in range(args.steps):
        f_d.copy_(f_h, non_blocking=True)
        x.zero_()
        ksp_mx.solve(x, f_d)
        x_h.copy_(x, non_blocking=True)
    e1.record()
    torch.cuda.synchronize()
    t_e2e = max_over_ranks(e0.elapsed_time(e1) / 1e3, ws)
    w_e2e = time.time() - w0

    mx_outer = statistics.mean(m.iter for m in mons)
    mx_inner = statistics.mean(m.inner_iter for m in mons)
    out = {
        "metric": METRIC,
        "value": round(ws * args.steps / t_mx, 4),
        "unit": "solves/s",
        "n_gpus": ws,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": round(t_mx / args.steps * 1e3, 3),
        "s_per_solve": round(t_mx / args.steps, 5),
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 inner / f64 outer",
        "data": "synthetic (seeded generators; no dataset)",
        "config": {"workload": f"{args.config}: {cfg['desc']}", "n_local_dofs": n, "n_unique_dofs": coef.nu,
                   "method": (f"cg_mixed (PCG in FP32 with the {args.pc_used} preconditioner, FP64 reliable "
                              f"updates at delta={args.delta:g})"
                              if args.method == "cg_mixed" else
                              f"fcg_mixed (inner Jacobi-PCG FP32 to {args.inner_rtol:g}, outer FCG(1) FP64)"),
                   "l2": "inputs larger than L2 (FP64 G 805 MB, FP32 G 403 MB at c2)",
                   "parallelism": "replicas only" if ws > 1 else "1 GPU"},
        "iterations": {"outer_mean": mx_outer, "inner_mean": mx_inner,
                       "fp64_ax_per_solve": mons[-1].fp64_ax},
        "fp64_dropin": {"s_per_solve": round(t64 / args.fp64_steps, 5), "iters": mons64[-1].iter,
                        "status": mons64[-1].status},
        "speedup_vs_fp64_dropin": round((t64 / args.fp64_steps) / (t_mx / args.steps), 3),
        "error_vs_fp64_solution": err_vs_fp64,
        "ax_gdof_s": {"fp64": round(n / t_ax64 / 1e9, 3), "fp32": round(n / t_ax32 / 1e9, 3)},
        "roofline": roof,
        "roofline_fp64_ax": roof64,
        "kernels_in_one_solve": ktimes,
        "e2e": {"value": round(ws * args.steps / t_e2e, 4), "unit": "solves/s",
                "h2d_bytes_per_step": int(f_h.numel() * 8), "d2h_bytes_per_step": int(x_h.numel() * 8),
                "wall_s": round(w_e2e, 4)},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "setup_s": round(t_setup, 3),
    }
    # CPU baseline: the oracle on this host, rank 0 at N=1 only
    if rank == 0 and ws == 1 and not args.no_cpu:
        out["cpu_baseline"] = cpu_sample(cfg, args.cpu_iters, mons64[-1].iter)
    return out


# ---------------------------------------------------------------------------
# CPU (reference algorithm) arm
# ---------------------------------------------------------------------------
def setup_cpu_case(cfg):
    import numpy as np
    from oracle import oracle as orc
    orc.build()
    ex, ey, ez = cfg["E"]
    m = orc.build_mesh(ex, ey, ez, LX, amp=cfg["amp"], seed=MESH_SEED)
    mask = orc.mask_face_xmax(ex, ey, ez, LX) if cfg["dirichlet"] else None
    h1c, h2 = 1.0, None
    if cfg["case"] == "poisson_fourier":
        k, a, ph = orc.fourier_params(RHS_SEED, 16)
        f = orc.assemble_rhs(m, orc.field_fourier(m, k, a, ph), mask)
    elif cfg["case"] == "brinkman_blobs":
        rho = orc.field_blobs(m, RHO_SEED, 12, 0.1)
        h2 = orc.ramp_forward(1.0 - rho, 0.0, 1e4, 8.0, 0)
        h1c = 0.01
        k, a, ph = orc.fourier_params(RHS_SEED, 16)
        f = orc.assemble_rhs(m, orc.field_fourier(m, k, a, ph), mask)
    else:
        rho = orc.field_uniform(m, RHO_SEED, 2, 0.0, 1.0)
        h2 = orc.ramp_forward(1.0 - rho, 0.0, 1e4, 8.0, 0)
        b = orc.field_uniform(m, RHS_SEED, 3, -1.0, 1.0)
        f = b - np.sum(b * m.mult) / m.nu
    dinv = orc.jacobi(m, h1c=h1c, h2=h2, mask=mask)
    return orc, m, mask, h1c, h2, f, dinv


def reference_iterations(config):
    """Iterations of the oracle's FP64 Jacobi-PCG to 1e-10 on `config`, as
    recorded by a full run (oracle/iterations.json), or None."""
    try:
        return int(json.load(open(os.path.join(ROOT, "oracle", "iterations.json")))[config]["iters"])
    except Exception:
        return None


def cpu_sample(cfg, iters, solve_iters):
    orc, m, mask, h1c, h2, f, dinv = setup_cpu_case(cfg)
    t_it = orc.cg_time_per_iter(m, f, iters, h1c=h1c, h2=h2, mask=mask, dinv=dinv)
    s_solve = t_it * solve_iters
    return {"value": round(1.0 / s_solve, 5), "unit": "solves/s", "cores": orc.num_threads(), "kind": "port",
            "s_per_solve": round(s_solve, 3), "s_per_iter": round(t_it, 5),
            "sample": f"{iters} FP64 Jacobi-PCG iterations of the same case on {orc.num_threads()} host threads, "
                      f"scaled by the {solve_iters} iterations of the FP64 solve to 1e-10"}


def setup_cpu_sequence(name, t):
    """The oracle's copy of solve t of a sequence: mesh, mask, h2 = chi of
    that solve's design, and its right-hand side."""
    import numpy as np
    from oracle import oracle as orc
    orc.build()
    cfg = SEQUENCES[name]
    ex, ey, ez = cfg["E"]
    m = orc.build_mesh(ex, ey, ez, LX, lo=cfg["lo"], hi=cfg["hi"], amp=cfg["amp"], seed=MESH_SEED)
    mask = orc.mask_face_xmax(ex, ey, ez, LX)
    rho = orc.field_blobs(m, RHO_SEED, 12, 0.1)
    for q in range(1, t // DESIGN_EVERY + 1):
        d = orc.field_fourier(m, *orc.fourier_params(1000 + q, 8))
        rho = np.clip(rho + 0.01 * d / np.abs(d).max(), 0.0, 1.0)
    h2 = orc.ramp_forward(1.0 - rho, 0.0, 1e4, 8.0, 0)
    import __graft_entry__ as ge  # the AR(1) parameters (host code, no GPU)
    k, ph, amps = ge.load_package().ar1_modes(RHS_SEED, 32, cfg["nsolves"], rho=0.98)
    f = orc.assemble_rhs(m, orc.field_fourier(m, k.reshape(-1, 3), amps[t], ph), mask)
    dinv = orc.jacobi(m, h1c=1.0, h2=h2, mask=mask)
    return orc, m, mask, h2, f, dinv


def sequence_fp64_iterations(name):
    """Iterations per solve of the plain FP64 drop-in (Jacobi-PCG + residual
    projection) on the timed solves of the sequence, as recorded from the
    drop-in's run on the GPU (the same algorithm as the oracle's CG; the
    parity tests hold the two iteration counts within 2)."""
    try:
        return float(json.load(open(os.path.join(ROOT, "oracle", "iterations.json")))[name + "seq"]["iters"])
    except Exception:
        return None


def cpu_sample_seq(name, iters, solve_iters):
    t = SEQUENCES[name]["ntrain"]
    orc, m, mask, h2, f, dinv = setup_cpu_sequence(name, t)
    t_it = orc.cg_time_per_iter(m, f, iters, h1c=1.0, h2=h2, mask=mask, dinv=dinv)
    if solve_iters is None:
        solve_iters = sequence_fp64_iterations(name)
    s_solve = t_it * solve_iters if solve_iters else None
    return {"value": round(1.0 / s_solve, 6) if s_solve else None, "unit": "solves/s", "cores": orc.num_threads(),
            "kind": "port", "s_per_iter": round(t_it, 4), "s_per_solve": round(s_solve, 2) if s_solve else None,
            "sample": f"{iters} FP64 Jacobi-PCG iterations of solve {t + 1} of the sequence (the oracle, "
                      f"{orc.num_threads()} host threads), times the {solve_iters} iterations per solve of the FP64 "
                      f"drop-in on the timed solves"}


def run_reference_sequence(args, ws, rank):
    """The reference algorithm on the host cores for the sequence workload:
    FP64 Jacobi-PCG (the oracle, all host threads).  Each step times
    --cpu-iters CG iterations of the first evaluation solve; ms_per_step is
    that measured time.  `value` (solves/s) scales the time per iteration by
    the iterations per solve of the FP64 drop-in (iterations_scaling says
    which).  A full CPU solve of C1 (8^3 elements) is timed outright
    beside it."""
    if rank != 0:
        return None
    import numpy as np
    name = args.config_seq
    t = SEQUENCES[name]["ntrain"]
    t_set = time.time()
    orc, m, mask, h2, f, dinv = setup_cpu_sequence(name, t)
    t_set = time.time() - t_set
    for _ in range(max(args.warmup, 1)):
        orc.cg_time_per_iter(m, f, 1, h1c=1.0, h2=h2, mask=mask, dinv=dinv)
    samples = [orc.cg_time_per_iter(m, f, args.cpu_iters, h1c=1.0, h2=h2, mask=mask, dinv=dinv)
               for _ in range(args.steps)]
    t_it = statistics.median(samples)
    iters = sequence_fp64_iterations(name)
    s_solve = t_it * iters if iters else None
    val = round(1.0 / s_solve, 7) if s_solve else None
    cores = orc.num_threads()
    del m, f, dinv, h2
    # one CPU solve timed outright: C1 (8^3 affine, N=7, Brinkman RAMP, Jacobi-PCG to 1e-10)
    orc1, m1, mask1, h1c1, h21, f1, dinv1 = setup_cpu_case(CONFIGS["c1"])
    t1 = time.time()
    _, it1, r01, r11 = orc1.cg(m1, f1, h1c=h1c1, h2=h21, mask=mask1, dinv=dinv1, rtol=RTOL, max_iter=20000)
    t1 = time.time() - t1
    sample = (f"each step: {args.cpu_iters} FP64 Jacobi-PCG iterations of solve {t + 1} of the {name} sequence on "
              f"{cores} host threads (the oracle); value = 1 / (median time per iteration x {iters} iterations per "
              f"solve of the FP64 drop-in)")
    return {
        "metric": METRIC, "impl": "reference", "value": val, "unit": "solves/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(t_it * args.cpu_iters * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded generators; no dataset)",
        "config": {"workload": f"{name}seq sequence: {SEQUENCES[name]['desc']}",
                   "n_local_dofs": int(np.prod(SEQUENCES[name]["E"])) * LX ** 3,
                   "method": "FP64 Jacobi-PCG, matrix-free sum factorisation (C oracle, OpenMP)"},
        "iterations_scaling": {"timed_per_step": args.cpu_iters, "iterations_per_solve": iters,
                               "source": "FP64 drop-in (Jacobi-PCG + projection) on the timed solves, oracle/iterations.json",
                               "s_per_iter": round(t_it, 4), "s_per_solve": round(s_solve, 2) if s_solve else None},
        "c1_full_solve": {"s": round(t1, 3), "iterations": it1, "res_start": r01, "res_final": r11,
                          "solves_per_s": round(1.0 / t1, 3), "cores": cores},
        "setup_s": round(t_set, 2),
        "cpu_baseline": {"value": val, "unit": "solves/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def run_reference(args, ws, rank):
    if rank != 0:
        return None
    cfg = CONFIGS[args.config]
    t0 = time.time()
    orc, m, mask, h1c, h2, f, dinv = setup_cpu_case(cfg)
    t_setup = time.time() - t0
    # iteration count of the full solve to 1e-10: measured once with this
    # same oracle (oracle/iterations.json records the run), else solved here
    t_full = None
    known = reference_iterations(args.config)
    if known is not None:
        iters = known
    else:
        t0 = time.time()
        _, iters, r0, r1 = orc.cg(m, f, h1c=h1c, h2=h2, mask=mask, dinv=dinv, rtol=RTOL, max_iter=20000)
        t_full = time.time() - t0
    for _ in range(max(args.warmup - 1, 0)):
        orc.cg_time_per_iter(m, f, 2, h1c=h1c, h2=h2, mask=mask, dinv=dinv)
    samples = []
    for _ in range(args.steps):
        samples.append(orc.cg_time_per_iter(m, f, args.cpu_iters, h1c=h1c, h2=h2, mask=mask, dinv=dinv))
    t_it = statistics.median(samples)
    s_solve = t_it * iters
    val = round(1.0 / s_solve, 5)
    cores = orc.num_threads()
    how = (f"timed once here: {t_full:.2f} s" if t_full is not None else
           "iteration count of the oracle's full solve recorded in oracle/iterations.json")
    sample = (f"each step: {args.cpu_iters} FP64 Jacobi-PCG iterations of the {args.config} case on {cores} host "
              f"threads, scaled by the {iters} iterations of a full solve to 1e-10 ({how})")
    return {
        "metric": METRIC, "impl": "reference", "value": val, "unit": "solves/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(s_solve * 1e3, 3),
        "s_per_solve": round(s_solve, 4), "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded generators; no dataset)",
        "config": {"workload": f"{args.config}: {cfg['desc']}", "n_local_dofs": m.n, "n_unique_dofs": m.nu,
                   "method": "FP64 Jacobi-PCG, matrix-free sum factorisation (C oracle, OpenMP)"},
        "iterations": iters, "full_solve_s": None if t_full is None else round(t_full, 3),
        "setup_s": round(t_setup, 3),
        "cpu_baseline": {"value": val, "unit": "solves/s", "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": val, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main(argv=None):
    p = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--config", choices=sorted(CONFIGS) + [k + "seq" for k in SEQUENCES], default="c5seq",
                   help="c5seq (default, the headline): the 64^3 Brinkman sequence with the learned guess; "
                        "c1/c2/c3/c5: single solves from a zero guess")
    p.add_argument("--method", choices=["cg_mixed", "fcg_mixed"], default="cg_mixed")
    p.add_argument("--delta", type=float, default=None,
                   help="reliable-update threshold of cg_mixed (default: 2.2e-4 with schwarz2, 0.1 otherwise)")
    p.add_argument("--pc", choices=["auto", "jacobi", "schwarz", "schwarz2"], default="auto",
                   help="FP32 preconditioner of cg_mixed (auto: two-level Schwarz for Poisson, Jacobi for Brinkman)")
    p.add_argument("--fdm-path", type=int, default=0, choices=[0, 1, 2],
                   help="Schwarz FDM kernel: 0 FP32 even-odd (default), 1 tensor cores, 2 FP32 full products")
    p.add_argument("--mass-term", action="store_true",
                   help="Schwarz: additive diagonal term for the Brinkman mass part")
    p.add_argument("--inner-rtol", type=float, default=1e-4)
    p.add_argument("--inner-max", type=int, default=2000)
    p.add_argument("--fp64-steps", type=int, default=2)
    p.add_argument("--cpu-iters", type=int, default=None,
                   help="CG iterations per CPU sample (default: 2 for sequences, 20 for single solves)")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    p.add_argument("--kernels-only", action="store_true",
                   help="set up the workload and launch each hot kernel a few times (profiler captures)")
    p.add_argument("--traffic", type=float, default=None,
                   help="dram bytes per FP32 Ax launch from an ncu capture (reported as roofline.traffic)")
    p.add_argument("--sequence", choices=sorted(SEQUENCES), default=None,
                   help="instead of the headline line: a solve sequence with each initial-guess mode")
    p.add_argument("--fp64-sample", type=int, default=None,
                   help="FP64 drop-in solves sampled (default: 2 in the headline sequence, 10 in --sequence)")
    p.add_argument("--fp64-warm", type=int, default=8, help="FP64 solves before the sample (fills projection)")
    p.add_argument("--proj-l", type=int, default=20, help="projection space size of --sequence (Neko's default 20)")
    p.add_argument("--mma", action="store_true", help="time MMA design updates on the workload's DOF count")
    p.add_argument("--fp64-peak", action="store_true", help="measure the FP64 FMA roof (the FP64 denominator)")
    p.add_argument("--terms", action="store_true",
                   help="time the FP64 terms either side of each solve (residuals, advection, forcing)")
    p.add_argument("--seq-modes", default="zero,projection,learned,learned_only",
                   help="initial-guess modes of --sequence (comma separated)")
    p.add_argument("--guess", default="learned_only", choices=["zero", "projection", "learned", "learned_only"],
                   help="initial-guess mode of the headline sequence (learned_only: the network's guess as x0, "
                        "behind the zero-guess guard; learned: the guess as an extra projection direction)")
    p.add_argument("--train-steps", type=int, default=30, help="Adam steps per training solve")
    p.add_argument("--short-eval", action="store_true",
                   help="headline sequence: skip the untimed rest of the evaluation half")
    p.add_argument("--no-compare", action="store_true",
                   help="headline sequence: skip the projection-only and zero-guess runs of the timed solves")
    args = p.parse_args(argv)
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else max(args.warmup, 1)
    args.config_seq = args.config[:-3] if args.config.endswith("seq") else None
    if args.config_seq and (args.terms or args.mma or args.kernels_only or args.sequence or args.fp64_peak):
        args.config, args.config_seq = "c2", None  # the analysis modes run on a single-solve mesh
    if args.fp64_sample is None:
        args.fp64_sample = 2 if args.config_seq else 10
    if args.cpu_iters is None:
        args.cpu_iters = 2 if args.config_seq else 20
    ws, rank, local = dist_env()
    if args.sequence:
        print(json.dumps(run_sequence(args, local)), flush=True)
        return 0
    if args.terms:
        print(json.dumps(run_terms(args, local)), flush=True)
        return 0
    if args.mma:
        print(json.dumps(run_mma(args, local)), flush=True)
        return 0
    if args.fp64_peak:
        import ctypes as C
        import torch
        import __graft_entry__ as ge
        torch.cuda.set_device(local)
        pkg = ge.load_package()
        probe = C.CDLL(os.path.join(ROOT, "neko-top_gb300", "lib", "libntgb300_probe.so"))
        probe.ntgprobe_fp64.restype = C.c_int
        probe.ntgprobe_fp64.argtypes = [C.c_int, C.POINTER(C.c_double), C.c_void_p]
        vals = []
        with ClockSampler(local) as clk:
            for _ in range(max(args.steps, 3)):
                tf = C.c_double()
                st = probe.ntgprobe_fp64(1 << 16, C.byref(tf), None)
                if st != 0:
                    raise RuntimeError(f"FP64 probe failed ({st})")
                vals.append(tf.value)
        print(json.dumps({"mode": "fp64_peak", "unit": "TFLOP/s", "runs": [round(v, 4) for v in vals],
                          "median": round(statistics.median(vals), 4), "clocks": clk.summary()}), flush=True)
        return 0
    if args.impl == "reference":
        res = run_reference_sequence(args, ws, rank) if args.config_seq else run_reference(args, ws, rank)
        if res is not None:
            print(json.dumps(res), flush=True)
        return 0
    if ws > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    res = run_headline_sequence(args, ws, rank, local) if args.config_seq else run_ours(args, ws, rank, local)
    if rank == 0:
        print(json.dumps(res), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

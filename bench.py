"""Benchmark: 256^3 pressure-Poisson solves per second on one GB300.

Workload (seeded synthetic inputs; the reference ships no decks): a 256^3 box
[0,1]^3 tanh-stretched toward the centre (beta 1.5) with a stationary
ghost-cell sphere (r = 0.15, 4x-subdivided icosphere, 5120 triangles); RHS =
divergence of a Gaussian random velocity field with |k| <= 8, mean removed and
made discretely compatible; one step = one solve_poisson from pPrime = 0 to
relative residual 1e-8 (max-norm <= 1e-8 max|nlu0|).  The headline arm is
the mixed-precision form (FP32 cycle inside FP64 refinement); the plain FP64
form is timed on the same inputs and reported beside it.

  value  : solves/s with pPrime/nlu0 resident in HBM (fsi_mg_solve_device),
           device time from CUDA events on the solver's stream.
  e2e    : solves/s through fsi_mg_solve with pinned HOST buffers, the H2D of
           pPrime and nlu0 and the D2H of pPrime inside the timed region.
  --impl reference : the reference MG algorithm (the C restatement in oracle/,
           serial like the reference, its own line order) timed on complete
           solves of the 128^3 config-2 workload, K solves as concurrent
           single-threaded replicas on the host cores.
  cpu_baseline : one complete 128^3 config-2 solve of the same oracle on one
           core, in the same run as the GPU's config-2 solves (config2 block:
           solves/s of four GPU forms, the timed ratios, and the parity of the
           converged pressures); a 256^3 figure is only reported as a labelled
           model (reference_model_256).

Multi-GPU: the path does not shard (replicas only); each rank runs its own
replica and value is the sum over ranks.
"""
from __future__ import annotations

import argparse
import copy
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "256³ Poisson solves/s @1e-8 resid, mixed vs FP64 GPU; HBM GB/s; adjoint/fwd"
PEAKS = ROOT / "MEASURED_PEAKS.json"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--tol", type=float, default=1e-8)
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--krylov", type=int, default=30, help="FGMRES restart length around MG_Solver (0: stationary)")
    ap.add_argument("--mgcycle", choices=("V", "W", "F"), default="V",
                    help="multigrid cycle of the headline forms (mgCycleX/Y/Z)")
    ap.add_argument("--iter-finest", type=int, default=1,
                    help="line sweeps per colour and direction on the finest levels of the headline forms "
                         "(iterFinest; the reference's input uses 2, the stationary forms keep it)")
    ap.add_argument("--omega", type=float, default=1.5,
                    help="line-SOR relaxation of the headline forms (omega; the reference's input uses 1, the "
                         "stationary forms keep it)")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-steps", action="store_true", help="skip the face_vel/correct_vel/update_pressure timing")
    ap.add_argument("--steps-only", action="store_true",
                    help="only the face_vel/correct_vel/update_pressure timing on the sphere grid (profiling)")
    ap.add_argument("--rollout", type=int, default=0,
                    help="run N fractional steps of the 192x128x128 sphere channel (Re 300, dt 0.005) and print "
                         "their line instead of the solve benchmark")
    ap.add_argument("--rollout-cells", type=int, nargs=3, default=(192, 128, 128))
    ap.add_argument("--rollout-adjoint", type=int, default=0,
                    help="with --rollout: the adjoint over the last N steps (checkpoints every 10)")
    ap.add_argument("--no-rollout", action="store_true",
                    help="skip the 200-step sphere-wake channel rollout reported beside the solve benchmark")
    ap.add_argument("--adjoint-n", type=int, default=96)
    ap.add_argument("--adjoint-dirs", type=int, default=200)
    ap.add_argument("--profile", action="store_true",
                    help="profiling driver: raw RHS, two outer iterations of each precision, no other work")
    ap.add_argument("--profile-krylov", action="store_true",
                    help="profiling driver: raw RHS, one mixed FGMRES solve capped at 6 MG applications")
    ap.add_argument("--profile-fp64", action="store_true",
                    help="profiling driver: one launch each of the FP64 kernels (face_vel_rhs, correct_vel, "
                         "rhs_advec_diff, calc_residual, a factored FP64 x sweep) and the DFMA roof on the sphere grid")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def job_seconds(local_seconds: float, world: int, device: str = "cuda") -> float:
    """The job's timed seconds: the maximum over ranks of each rank's timed
    seconds (each rank runs its own replica; one rank: its own time)."""
    if world <= 1:
        return local_seconds
    import torch
    t = torch.tensor([local_seconds], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world: int, steps: int, job_s: float) -> float:
    """Whole-job solves/s: every rank solved `steps` problems within job_s."""
    return world * steps / job_s


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.lines = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


def build_problem(n, seed, tol, solver_cls):
    from flow_structure_interaction_fem_ibm_gb300 import problem as P
    pr = P.sphere(n, seed=seed, stretch=1.5)
    # discrete compatibility shift from two GPU solves run to their residual plateau
    def stagnated(f):
        pp = copy.deepcopy(pr.params)
        pp.restol_Poisson, pp.precision_mode, pp.outer_krylov = 0.0, 1, 0

        def solve_from_zero(rhs, iters):
            pp.iterMax_Poisson = iters
            s = solver_cls(pp, pr.x, pr.y, pr.z).set_boundary(pr.geom)
            p0 = np.zeros(pr.shape, order="F")
            s.solve_poisson(p0, rhs)
            h = s.residual_history()
            s.close()
            return p0, h

        return P.stall_until_plateau(solve_from_zero, f, iters=150, rtol=1e-5)
    shift = P.make_compatible(pr, stagnated)
    pr.params.restol_Poisson = tol * float(np.abs(pr.nlu0).max())
    pr.params.iterMax_Poisson = 500
    return pr, shift


_ORACLE = {}


def oracle_iteration_time(n, seed, reps=1):
    """Seconds per outer iteration of the oracle (serial reference MG with the
    reference's line ordering, iRedBlack 0) at n^3: MG_Solver,
    GCM_correct_pressure and calc_residual, as in IBM/CORE_POISSON.F90:640-663.
    The oracle is built once per process."""
    from flow_structure_interaction_fem_ibm_gb300 import problem as P
    from oracle.oracle import Oracle
    key = (n, seed)
    if key not in _ORACLE:
        pr = P.sphere(n, seed=seed, stretch=1.5)
        o = Oracle(pr)
        p = np.zeros(pr.shape, order="F")
        o.subtract_average(p)
        _ORACLE[key] = (pr, o, p)
    pr, o, p = _ORACLE[key]
    t0 = time.perf_counter()
    for _ in range(reps):
        o.mg_solver(p, pr.nlu0)
        o.correct_pressure(p)
        o.calc_residual(p, pr.nlu0)
    return (time.perf_counter() - t0) / reps


# Outer iterations the reference's stationary solve_poisson needs on this
# workload (same recipe and compatibility shift, reference line ordering),
# measured with the oracle: the full solve is hours of serial CPU time at
# 256^3, so the timed CPU sample is one iteration and the count comes from here.
# (n, seed, tol): (iterations, how they were obtained)
REFERENCE_ITERATIONS = {
    (128, 3, 1e-8): (121, "oracle solve to convergence at 128^3 (reference line order, iRedBlack 0)"),
    (256, 3, 1e-8): (413, "160 oracle iterations run at 256^3 (reference line order; maxres 0.0199 against "
                          "restol 3.50e-6, 1.9 h on one core) and the remaining 253 extrapolated at the "
                          "asymptotic contraction 0.9664 per iteration, constant over the last 25 iterations"),
}


def _oracle_complete_solve(params_blob, x, y, z, geom, nlu0):
    """One complete solve_poisson of the oracle (serial C restatement of the
    reference MG, the reference's own lexicographic line order, iRedBlack 0)
    from pPrime = 0, timed end to end on this process's core."""
    from flow_structure_interaction_fem_ibm_gb300 import problem as P
    from oracle.oracle import Oracle
    pr = P.Problem(params_blob, x, y, z, geom, nlu0, "oracle_complete")
    pr.params.iRedBlack, pr.params.coarse_flag_mode = 0, 0
    t0 = time.perf_counter()
    o = Oracle(pr)
    t1 = time.perf_counter()
    r = o.solve()
    t2 = time.perf_counter()
    o.close()
    return {"p": r["p"], "status": r["status"], "iters": r["iters"], "maxres": r["maxres"],
            "setup_s": t1 - t0, "solve_s": t2 - t1}


def _oracle_worker(inbox, outbox):
    """Spawned before the first GPU call: runs the oracle jobs the main process
    sends (the CPU side of the same run) on its own core."""
    while True:
        job = inbox.get()
        if job is None:
            return
        kind, payload = job
        try:
            if kind == "complete":
                outbox.put((kind, _oracle_complete_solve(*payload)))
            elif kind == "iteration":
                n, seed = payload
                oracle_iteration_time(n, seed)   # builds the oracle state (not timed)
                outbox.put((kind, {"n": n, "seconds": oracle_iteration_time(n, seed)}))
        except Exception as e:   # reported in the bench line, never hides a GPU result
            outbox.put((kind, {"error": repr(e)}))


class OracleJobs:
    """Two spawned CPU workers (one core each) for the oracle work that runs
    beside the GPU benchmark: the complete 128^3 solve and one 256^3 outer
    iteration."""

    def __init__(self, n_workers=2):
        import multiprocessing as mp
        ctx = mp.get_context("spawn")
        self.workers = []
        for _ in range(n_workers):
            inbox, outbox = ctx.Queue(), ctx.Queue()
            proc = ctx.Process(target=_oracle_worker, args=(inbox, outbox), daemon=True)
            proc.start()
            self.workers.append((proc, inbox, outbox))

    def submit(self, w, kind, payload):
        self.workers[w][1].put((kind, payload))

    def result(self, w, timeout=None):
        kind, res = self.workers[w][2].get(timeout=timeout)
        return res

    def close(self):
        for proc, inbox, _ in self.workers:
            inbox.put(None)
        for proc, _, _ in self.workers:
            proc.join(timeout=10)
            if proc.is_alive():
                proc.terminate()


def profile_traffic(n):
    """DRAM bytes per launch of the level-1 FP32 line relaxation from the
    committed ncu summary for this grid (None when there is none)."""
    import re
    f = ROOT / "profiles" / f"line_relaxation_fp32_{n}.md"
    if not f.exists():
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", f.read_text())
    return float(m.group(1)) if m else None


# Discrete compatibility shifts of the config-2 workload (128^3 stretched
# sphere, seed 2), from two FP64 plateau solves of the oracle on the current
# geometry (problem.compatibility_shift, plateau to 1e-10 relative; the value
# the GPU arm computes for itself and prints as config2.compat_shift agrees to
# its mixed-precision plateau).  The reference arm runs no GPU code, so it
# takes the shift from here; the shift is a property of the discrete operator
# and the right-hand side, not of the solver.  It must follow the geometry:
# an error dc leaves a residual floor of about 51 dc in max-norm, against a
# tolerance of 1.9e-6.
CONFIG2_SHIFT = {1e-8: -0.0003587849847243156}
# Digest of the config-2 inputs that shift belongs to (config2_digest); a CPU
# test compares it with the current geometry so that a geometry change cannot
# leave a stale shift behind.
CONFIG2_DIGEST = "de9188c1e263b9d8"


def config2_digest():
    """Digest of the config-2 workload's inputs: iblank, ghost list, stencil
    cells, image-point weights (to 1e-10) and the mean-free right-hand side
    (to 1e-8 of its scale)."""
    import hashlib
    from flow_structure_interaction_fem_ibm_gb300 import problem as P
    pr = P.sphere(128, seed=2, stretch=1.5)
    g = pr.geom
    scale = float(np.abs(pr.nlu0).max())
    h = hashlib.sha256()
    for a in (g.iblank, g.iG, g.jG, g.kG, g.iCI, g.jCI, g.kCI, np.round(g.coeff, 10),
              np.round(pr.nlu0 / scale, 8)):
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()[:16]


def config2_problem(tol, shift=None, solver_cls=None):
    """Config 2: 128^3 [0,1]^3 tanh-stretched (beta 1.5) with the r = 0.15
    ghost-cell sphere, Gaussian |k| <= 8 right-hand side (seed 2), mean
    removed and made discretely compatible, restol = tol max|nlu0|."""
    from flow_structure_interaction_fem_ibm_gb300 import problem as P
    if shift is None:
        pr, shift = build_problem(128, 2, tol, solver_cls)
        return pr, shift
    pr = P.sphere(128, seed=2, stretch=1.5)
    pr.nlu0 += shift * P.fluid_indicator(pr)
    pr.params.restol_Poisson = tol * float(np.abs(pr.nlu0).max())
    # the oracle needs 133 iterations; the bound keeps a solve that cannot reach the
    # tolerance (a compatibility shift that no longer fits the geometry) to minutes
    pr.params.iterMax_Poisson = 500
    return pr, shift


def _reference_replica(job):
    """One replica of the reference arm: warm-up outer iterations (untimed),
    then its share of the complete solves, each timed end to end."""
    tol, shift, warm_iters, nsolve, ready, start_evt = job
    from oracle.oracle import Oracle
    pr, _ = config2_problem(tol, shift)
    pr.params.iRedBlack, pr.params.coarse_flag_mode = 0, 0
    if warm_iters > 0:
        q = copy.deepcopy(pr)
        q.params.iterMax_Poisson, q.params.restol_Poisson = warm_iters, 0.0
        Oracle(q).solve()
    o = Oracle(pr)   # MG_initial and the geometry hand-over happen once, outside the timed solves
    ready.put(1)
    start_evt.wait()
    out = []
    for _ in range(nsolve):
        t0 = time.perf_counter()
        r = o.solve()
        out.append({"seconds": time.perf_counter() - t0, "iters": r["iters"], "status": r["status"],
                    "end": time.time()})
    o.close()
    return out


def profile_fp64_instr():
    """FP64-pipe thread-instructions per interior cell of the FP64 kernels,
    from the committed ncu summary (profiles/fp64_kernels_160.md); {} when
    absent."""
    import re
    f = ROOT / "profiles" / "fp64_kernels_160.md"
    if not f.exists():
        return {}
    return {m.group(1): float(m.group(2))
            for m in re.finditer(r"fp64_instr_per_cell\s+(\w+):\s*([0-9.eE+]+)", f.read_text())}


def run_reference(args, rank, world):
    """The reference arm: the oracle (serial C restatement of the reference's
    MG, its own lexicographic line order) timed on complete solves of the
    config-2 workload on the host cores.  The K timed steps are K complete
    solves run as concurrent single-threaded replicas (at most one process per
    solve); value = K / wall time of the timed region."""
    if rank != 0:
        print(json.dumps({"impl": "reference", "rank": rank, "skipped": True}), file=sys.stderr)
        return
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    key = args.tol
    if key not in CONFIG2_SHIFT:
        print(json.dumps({"impl": "reference", "unavailable": f"no recorded compatibility shift for tol {key:g}"}))
        return
    shift = CONFIG2_SHIFT[key]
    nproc = max(1, min(args.steps, 2 * cores))
    share = [args.steps // nproc + (1 if i < args.steps % nproc else 0) for i in range(nproc)]
    ctx = mp.get_context("spawn")
    t_all = time.perf_counter()
    with ctx.Manager() as mgr:
        start, ready = mgr.Event(), mgr.Queue()
        with ctx.Pool(nproc) as pool:
            res = pool.map_async(_reference_replica,
                                 [(args.tol, shift, args.warmup, k, ready, start) for k in share])
            # every replica builds its state and runs its warm-up iterations, then waits for the start
            for _ in range(nproc):
                ready.get(timeout=1200)
            t0 = time.time()
            start.set()
            runs = [r for part in res.get() for r in part]
    wall = max(r["end"] for r in runs) - t0
    ok = all(r["status"] == 0 for r in runs)
    value = args.steps / wall
    per = [r["seconds"] for r in runs]
    out = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * wall / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"sphere_128^3_tanh1.5_r0.15_seed2_tol{args.tol:g} (config 2)", "grid": 128,
                   "tol": args.tol, "compat_shift": shift,
                   "parallelism": f"{nproc} concurrent single-threaded replicas on {cores} host cores",
                   "same_config_as_gpu_arm": False,
                   "why": "a complete 256^3 solve of the reference takes hours on one core; the GPU arm's "
                          "line carries its own 128^3 config-2 solves timed beside one complete oracle solve"},
        "cpu_baseline": {"value": value, "unit": "solves/s", "cores": min(nproc, cores), "kind": "port",
                         "sample": (f"{args.steps} complete solve_poisson runs of the 128^3 config-2 workload "
                                    f"(oracle, reference line order, tol {args.tol:g}) as concurrent replicas; "
                                    f"warm-up: {args.warmup} outer iterations per replica, untimed")},
        "e2e": {"value": value, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "solve_seconds": {"min": min(per), "median": float(np.median(per)), "max": max(per)},
        "iters": sorted({r["iters"] for r in runs}), "all_converged": ok,
        "wall_s": time.perf_counter() - t_all,
    }
    print(json.dumps(out))


def adjoint_check(n, ndir, h=1e-6):
    """Projection-step adjoint on the n^3 uniform grid with the r = 0.15 sphere:
    velocity = seeded Gaussian field (|k| <= 8, seed 4), loss = kinetic energy
    of the projected field in [0.6,0.9]x[0.35,0.65]^2.  Times one forward and
    one backward (GPU synchronised, wall clock: the adjoint is a torch harness
    around the multigrid) and checks the gradient against FP64 central
    differences on `ndir` seeded random directions."""
    import torch
    from flow_structure_interaction_fem_ibm_gb300 import problem as P
    from flow_structure_interaction_fem_ibm_gb300.adjoint import Projection, box_kinetic_energy
    pr = P.sphere(n, seed=4, stretch=None)
    t0 = time.perf_counter()
    proj = Projection(pr, "cuda")
    setup = time.perf_counter() - t0
    rng = np.random.Generator(np.random.PCG64(4))
    u, v, w = [torch.as_tensor(np.asfortranarray(P.gaussian_field(pr.params, pr.x, pr.y, pr.z, rng, 8)),
                               device="cuda") for _ in range(3)]
    fwd, bwd = [], []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        un, vn, wn, _ = proj.forward(u, v, w)
        torch.cuda.synchronize()
        fwd.append(time.perf_counter() - t0)
        outs = [t.detach().requires_grad_() for t in (un, vn, wn)]
        lam = torch.autograd.grad(box_kinetic_energy(pr, *outs), outs)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        gu, gv, gw = proj.backward(*lam)
        torch.cuda.synchronize()
        bwd.append(time.perf_counter() - t0)
    stats = dict(proj.stats)
    g = torch.Generator().manual_seed(11)
    loss = lambda a, b, c: float(box_kinetic_energy(pr, *proj.forward(a, b, c)[:3]))
    worst = 0.0
    for _ in range(ndir):
        d = [torch.randn(pr.shape[::-1], dtype=torch.float64, generator=g).permute(2, 1, 0).cuda() for _ in range(3)]
        fd = (loss(u + h * d[0], v + h * d[1], w + h * d[2]) - loss(u - h * d[0], v - h * d[1], w - h * d[2])) / (2 * h)
        an = float((gu * d[0]).sum() + (gv * d[1]).sum() + (gw * d[2]).sum())
        worst = max(worst, abs(fd - an) / abs(an))
    proj.close()
    f_s, b_s = float(np.median(fwd)), float(np.median(bwd))
    return {"config": f"sphere_{n}^3_uniform_r0.15_seed4_box_KE", "forward_s": f_s, "backward_s": b_s,
            "adjoint_over_forward": b_s / f_s, "forward_mg_applications": stats.get("forward_applications"),
            "transposed_mg_applications": stats.get("transposed_applications"), "fd_directions": ndir,
            "fd_h": h, "fd_worst_rel": worst, "setup_s": setup,
            "timing": "wall clock with the GPU synchronised, median of 3"}


def projection_steps(solver, pr, peak, reps=20):
    """The fractional-step routines either side of the solve on device arrays of
    the bench grid (face_vel + rhs_poisson, correct_vel, update_pressure; both
    frac_step_type branches): per kernel the device time of a replayed launch
    (CUDA events on the library's stream, fsi_mg_time_kernel 6/7/8), its
    algorithmic bytes and the fraction of the measured HBM bandwidth, and the
    wall time of one synchronous C-ABI call."""
    import torch
    rng = torch.Generator(device="cuda").manual_seed(17)
    sh = pr.shape[::-1]
    r = lambda: torch.randn(sh, dtype=torch.float64, device="cuda", generator=rng)
    u, v, w, p, pp = r(), r(), r(), r(), r()
    faces = [torch.zeros(sh, dtype=torch.float64, device="cuda") for _ in range(3)]
    nlu0 = torch.zeros(sh, dtype=torch.float64, device="cuda")
    fp = [t.data_ptr() for t in faces]
    torch.cuda.synchronize()   # the library's stream does not wait for torch's
    out = {}
    for frac, tag in ((0, "no_van_kan"), (1, "van_kan")):
        calls = {
            "face_vel_rhs": lambda: solver.face_vel_rhs(1e-3, u.data_ptr(), v.data_ptr(), w.data_ptr(), *fp,
                                                        nlu0.data_ptr(), frac_step_type=frac, d_p=p.data_ptr()),
            "correct_vel": lambda: solver.correct_vel(1e-3, pp.data_ptr(), u.data_ptr(), v.data_ptr(),
                                                      w.data_ptr(), *fp),
            "update_pressure": lambda: solver.update_pressure(pp.data_ptr(), p.data_ptr(), frac),
        }
        res = {}
        for which, (name, call) in zip((6, 7, 8), calls.items()):
            if frac == 1 and name == "correct_vel":
                continue   # correct_vel has no frac_step_type branch
            call()
            t0 = time.perf_counter()
            for _ in range(5):
                call()
            wall_us = (time.perf_counter() - t0) / 5 * 1e6
            ms, nb = solver.time_kernel(which, 0, reps)
            gbs = nb / (ms * 1e-3) / 1e9
            res[name] = {"device_us": 1e3 * ms, "alg_bytes": nb, "achieved_gbs": gbs, "frac": gbs / peak,
                         "call_wall_us": wall_us}
        out[tag] = res
    # momentum right-hand side (rhs_advec_diff, Crank-Nicolson, constant viscosity array, no bc arrays)
    visc = torch.full(sh, 1e-3, dtype=torch.float64, device="cuda")
    nl = [torch.zeros(sh, dtype=torch.float64, device="cuda") for _ in range(3)]
    torch.cuda.synchronize()
    solver.rhs_advec_diff(1e-3, [u.data_ptr(), v.data_ptr(), w.data_ptr()], fp, visc.data_ptr(),
                          [t.data_ptr() for t in nl], advec_scheme=2)
    ms, nb = solver.time_kernel(9, 0, reps)
    gbs = nb / (ms * 1e-3) / 1e9
    out["rhs_advec_diff_cn"] = {"device_us": 1e3 * ms, "alg_bytes": nb, "achieved_gbs": gbs, "frac": gbs / peak}
    del visc, nl
    # FP64 pipe roof on this GPU: independent DFMA chains on every SM (CUDA events, no settings changed)
    ms, flops = solver.time_kernel(10, 0, 10)
    out["fp64_roof"] = {"tflops": flops / (ms * 1e-3) / 1e12, "ms": ms, "flops_per_launch": flops,
                        "method": "k_dfma_peak: 4 independent DFMA chains x 4096 per thread, 8 CTAs of 256 per SM"}
    out["note"] = ("device_us: the routine's kernels (face_vel_rhs: shell zeroing, [uTilde], faces+divergence, "
                   "sum) replayed 20x; alg_bytes: FP64 fields read/written once per interior cell, no bc arrays; "
                   "update_pressure without its ghost-cell rows")
    del u, v, w, p, pp, faces, nlu0
    return out


def device_time_step(n, seed, tol, krylov, steps=3, reinv=1e-3, dt=1e-3):
    """One fractional time step kept in HBM through the C ABI, on the n^3
    stretched box without a body (its face_vel right-hand side is compatible),
    in the reference's order (IBM/CORE_TIME_STEP.F90:201-267):
    fsi_mg_rhs_advec_diff (Crank-Nicolson) -> fsi_mg_rhs_adjust_bc ->
    fsi_mg_solve_ad -> fsi_mg_face_vel_rhs -> fsi_mg_solve_device (mixed,
    FGMRES) -> fsi_mg_correct_vel -> fsi_mg_update_pressure, no host copy of a
    field.  Every timed step starts from the same state.  Wall time per routine
    (each call waits for its work), and the size-independent check of the
    step: the corrected face velocities are divergence-free to the solver's
    residual, max |div(face)/dt| over the interior <= restol (the face
    gradient of correct_vel and the Poisson operator are the same stencil)."""
    import torch
    from flow_structure_interaction_fem_ibm_gb300 import problem as P
    from flow_structure_interaction_fem_ibm_gb300.grid import Metrics
    from flow_structure_interaction_fem_ibm_gb300.poisson import PoissonSolver
    pr = P.box3d(n, seed=seed, stretch=1.5)
    q = copy.deepcopy(pr.params)
    q.restol_Poisson = tol * float(np.abs(pr.nlu0).max()) / dt
    q.iterMax_Poisson, q.precision_mode, q.outer_krylov = 400, 1, krylov
    q.restol_ad, q.iterMax_ad = 1e-10, 200
    s = PoissonSolver(q, pr.x, pr.y, pr.z).set_boundary(pr.geom)
    sh = pr.shape[::-1]
    g = torch.Generator(device="cuda").manual_seed(seed)
    z = lambda: torch.zeros(sh, dtype=torch.float64, device="cuda")
    u0, v0, w0 = (torch.randn(sh, dtype=torch.float64, device="cuda", generator=g) for _ in range(3))
    u, v, w = z(), z(), z()
    faces, faces0 = [z() for _ in range(3)], [z() for _ in range(3)]
    nl = [z() for _ in range(3)]
    nlu0, pp, p = z(), z(), z()
    visc = torch.full(sh, reinv, dtype=torch.float64, device="cuda")
    fp = [t.data_ptr() for t in faces]
    vp = [u.data_ptr(), v.data_ptr(), w.data_ptr()]
    nlp = [t.data_ptr() for t in nl]
    vis = [visc.data_ptr()] * 3
    # the previous step's face velocities (the library's stream does not wait for torch's)
    torch.cuda.synchronize()
    s.face_vel_rhs(dt, u0.data_ptr(), v0.data_ptr(), w0.data_ptr(), *[t.data_ptr() for t in faces0], nlu0.data_ptr())
    dinv = [torch.from_numpy(Metrics(c).dxinv).cuda() for c in (pr.x, pr.y, pr.z)]
    names = ["rhs_advec_diff", "rhs_adjust_bc", "solve_ad", "face_vel_rhs", "solve", "correct_vel",
             "update_pressure"]
    times = {k: [] for k in names}
    iters, ad_iters, worst = [], [], 0.0
    for it in range(steps + 1):
        u.copy_(u0); v.copy_(v0); w.copy_(w0); pp.zero_()
        for a, b in zip(faces, faces0):
            a.copy_(b)
        torch.cuda.synchronize()
        t = [time.perf_counter()]
        s.rhs_advec_diff(dt, vp, fp, visc.data_ptr(), nlp, bcvisc=vis, advec_scheme=2)
        t.append(time.perf_counter())
        s.rhs_adjust_bc(dt, fp, visc.data_ptr(), nlp, bcvisc=vis, advec_scheme=2)
        t.append(time.perf_counter())
        st_ad, nad, mr_ad = s.solve_ad(dt, fp, visc.data_ptr(), vp, nlp, bcvisc=vis, advec_scheme=2)
        t.append(time.perf_counter())
        s.face_vel_rhs(dt, *vp, *fp, nlu0.data_ptr())
        t.append(time.perf_counter())
        st, nit, mr, _, _ = s.solve_poisson_device(pp.data_ptr(), nlu0.data_ptr())
        t.append(time.perf_counter())
        s.correct_vel(dt, pp.data_ptr(), *vp, *fp)
        t.append(time.perf_counter())
        s.update_pressure(pp.data_ptr(), p.data_ptr(), 0)
        t.append(time.perf_counter())
        if st != 0 or st_ad != 0:
            raise RuntimeError(f"device time step: solve status {st} ({nit} iterations, maxres {mr}), "
                               f"solve_ad status {st_ad} ({nad} iterations, maxres {mr_ad})")
        if it == 0:
            continue   # warm-up (graph capture)
        for k, a_, b_ in zip(names, t[:-1], t[1:]):
            times[k].append(1e3 * (b_ - a_))
        iters.append(nit)
        ad_iters.append(nad)
        # (z, y, x) tensors: divergence of the corrected faces over the interior
        fu, fv, fw = faces
        I = slice(1, n + 1)
        div = ((fu[I, I, 2:n + 2] - fu[I, I, I]) * dinv[0][I].view(1, 1, -1)
               + (fv[I, 2:n + 2, I] - fv[I, I, I]) * dinv[1][I].view(1, -1, 1)
               + (fw[2:n + 2, I, I] - fw[I, I, I]) * dinv[2][I].view(-1, 1, 1)) / dt
        worst = max(worst, float(div.abs().max()))
    s.close()
    ms = {k: float(np.median(v_)) for k, v_ in times.items()}
    return {"workload": f"box3d_{n}^3_tanh1.5_no_body_Re{1 / reinv:g}_dt{dt:g}_CN_mixed_fgmres{krylov}",
            "steps": steps, "ms": ms, "step_ms": sum(ms.values()), "poisson_iters": iters,
            "solve_ad_iters": ad_iters, "restol": q.restol_Poisson, "restol_ad": q.restol_ad,
            "max_div_after_correction": worst, "divergence_free": worst <= q.restol_Poisson,
            "host_copies_per_step": 0}


def channel_rollout(steps, cells=(192, 128, 128), krylov=30, warmup=2, restol=1e-6, dt=0.005, re=300.0,
                    adjoint_steps=50, checkpoint_every=10, x_plane=3.0, mgcycle=1, pressure_guess="extrapolate",
                    iter_finest=1, omega=1.0):
    """The sphere-wake rollout: a 192 x 128 x 128 uniform channel on [0,6] x
    [0,4]^2, sphere of diameter 1 at (1.5, 2, 2) (GCM ghost cells), uniform
    inflow U = 1, zero-gradient outflow with the outflow mass balance,
    symmetry sides, Re 300, dt 0.005, Crank-Nicolson, mixed-precision
    pressure solve every step (FGMRES(krylov) around MG_Solver on the
    operator of the outflow compatibility fixed point; krylov 0: the
    stationary outer iteration), absolute tolerances restol (pressure) and
    1e-10 (momentum).  pressure_guess "extrapolate" starts each pressure
    solve from 2 p(n-1) - p(n-2) instead of the reference's p(n-1) (the same
    converged pressure to the tolerance; 17 instead of 21 applications per
    step on average over the first 100 steps).
    FractionalStep keeps every field in HBM; a step is one call per routine.
    Reports steps/s over the untimed steps after `warmup`, the per-stage wall
    time of one extra instrumented step, the solvers' iteration counts, the
    divergence of the corrected faces and the peak device memory.
    With adjoint_steps > 0 the rollout runs through step_adjoint.RolloutAdjoint
    (the same product step, with the state kept every checkpoint_every steps
    over the last adjoint_steps), then the adjoint of the loss "mean
    streamwise velocity in the cell plane nearest x = x_plane" back over those
    steps, its cost against the forward cost of the same steps, and one
    central-difference check of it on the product rollout."""
    import torch
    from flow_structure_interaction_fem_ibm_gb300 import problem as P
    from flow_structure_interaction_fem_ibm_gb300.grid import Metrics
    from flow_structure_interaction_fem_ibm_gb300.time_step import FractionalStep
    t0 = time.perf_counter()
    pr = P.channel(tuple(cells))
    q = pr.params
    q.precision_mode, q.outer_krylov = 1, krylov
    q.restol_Poisson, q.iterMax_Poisson = restol, 2000
    q.restol_ad, q.iterMax_ad = 1e-10, 200
    q.mgcycle = (mgcycle,) * 3
    q.iterFinest = iter_finest
    q.omega = omega
    inflow = np.array([[1.0, 0.0, 0.0]] + [[0.0, 0.0, 0.0]] * 5)
    fluid = 1.0 - pr.geom.iblank
    u0 = np.asfortranarray(fluid.astype(np.float64))
    zero = np.zeros(pr.shape, order="F")
    torch.cuda.reset_peak_memory_stats()
    free0, total = torch.cuda.mem_get_info()
    ra = None
    if adjoint_steps > 0:
        from flow_structure_interaction_fem_ibm_gb300.step_adjoint import RolloutAdjoint
        # transposed solves to 1e-10 (momentum) and 1e-9 (pressure) relative, the pressure one
        # preconditioned by a mixed-precision MG_Solver application, both warm-started from the
        # previous step's solution
        ra = RolloutAdjoint(pr, dt, 1.0 / re, inflow, advec_scheme=2, rtol_ad=1e-10, rtol_p=1e-9,
                            mixed_precondition=True, warm_start=True, pressure_guess=pressure_guess)
        fs = ra.fs
        setup_s = time.perf_counter() - t0
        ra.forward(u0, zero, zero, steps=warmup + steps, adjoint_steps=min(adjoint_steps, steps),
                   checkpoint_every=checkpoint_every, warmup=warmup)
        wall = ra.times["forward_s"]
        recs = ra.records[warmup:]
    else:
        fs = FractionalStep(pr, dt, 1.0 / re, inflow, advec_scheme=2, pressure_guess=pressure_guess).start(
            u0, zero, zero)
        setup_s = time.perf_counter() - t0
        for _ in range(warmup):
            fs.step()
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        recs = [fs.step() for _ in range(steps)]
        torch.cuda.synchronize()
        wall = time.perf_counter() - t1
    free_fwd, _ = torch.cuda.mem_get_info()
    lib_bytes = int(fs.s.stats()["device_bytes"])
    n = [c for c in cells]
    fu, fv, fw = fs.faces
    dinv = [torch.from_numpy(Metrics(c).dxinv).cuda() for c in (pr.x, pr.y, pr.z)]
    I, J, K = slice(1, n[0] + 1), slice(1, n[1] + 1), slice(1, n[2] + 1)
    fl = torch.from_numpy(np.ascontiguousarray(fluid.transpose())).cuda()[K, J, I]
    div = ((fu[K, J, 2:n[0] + 2] - fu[K, J, I]) * dinv[0][I].view(1, 1, -1)
           + (fv[K, 2:n[1] + 2, I] - fv[K, J, I]) * dinv[1][J].view(1, -1, 1)
           + (fw[2:n[2] + 2, J, I] - fw[K, J, I]) * dinv[2][K].view(-1, 1, 1)) * fl
    # the outflow cell layer (i = nx-1) carries div = -dt nlw0: its faces keep the zero-gradient
    # set_bc values while nlw0 adds the outflow pressure-gradient planes to the Poisson rows
    adiv = div.abs()
    am = int(torch.argmax(adiv))
    kk, rem = divmod(am, n[1] * n[0])
    jj, ii = divmod(rem, n[0])
    closure = (div + dt * fs.nlw0[K, J, I] * fl).abs()
    u = fs.vel[0]
    umax = float(u.abs().max())
    adjoint = None
    if ra is not None:
        adjoint = rollout_adjoint_report(pr, ra, x_plane)
    stage = fs.step(timed=True)
    free1, _ = torch.cuda.mem_get_info()
    out = {"profile": "channel_rollout",
           "workload": f"channel_{n[0]}x{n[1]}x{n[2]}_[0,6]x[0,4]^2_sphere_d1_at_(1.5,2,2)_Re{re:g}_dt{dt:g}_CN_"
                       f"mixed_{'fgmres' + str(krylov) if krylov else 'stationary'}_{'VWF'[mgcycle - 1]}cycle",
           "steps": steps, "warmup": warmup, "ms_per_step": 1e3 * wall / steps, "steps_per_s": steps / wall,
           "stage_ms": stage["ms"], "poisson_iters": [r["poisson_iters"] for r in recs],
           "ad_iters": [r["ad_iters"] for r in recs],
           "statuses_ok": all(r["poisson_status"] == 0 and r["ad_status"] == 0 for r in recs),
           "max_abs_div_after_correction": float(adiv.max()),
           "argmax_div_cell": [ii + 1, jj + 1, kk + 1],
           "max_abs_div_outside_outflow_layer": float(adiv[:, :, :-1].max()),
           "max_abs_div_plus_dt_nlw0": float(closure.max()),
           "divergence_note": "the maximum sits in the outflow cell layer, where div(face) = -dt nlw0 (the "
                              "reference's own chain gives the same, to 1e-12); div + dt nlw0 is the projection's "
                              "residual everywhere",
           "restol_Poisson": restol, "pressure_guess": pressure_guess, "iterFinest": iter_finest, "omega": omega,
           "mg_cycle": "VWF"[mgcycle - 1],
           "u_max": umax, "time": fs.time, "ghost_cells": int(pr.geom.nGhost),
           "device_bytes_in_use_forward": int(free0 - free_fwd), "device_bytes_in_use": int(free0 - free1),
           "torch_peak_bytes": int(torch.cuda.max_memory_allocated()),
           "library_bytes": lib_bytes, "setup_s": setup_s, "adjoint": adjoint}
    if ra is not None:
        ra.close()
    else:
        fs.close()
    return out


def rollout_adjoint_report(pr, ra, x_plane):
    """The adjoint of the last ra.adj steps of a finished RolloutAdjoint
    forward for L = mean streamwise velocity in the plane nearest x_plane,
    timed against the forward cost of the same steps, and one central
    difference of L on the product rollout in a random direction of the
    velocities at the first adjoint step."""
    import torch
    from flow_structure_interaction_fem_ibm_gb300.step_adjoint import wake_plane_loss
    loss_fn = lambda vel: wake_plane_loss(pr, vel[0], x_plane)[0]
    torch.cuda.reset_peak_memory_stats()
    L, cot = ra.gradient(loss_fn)
    adj_peak = int(torch.cuda.max_memory_allocated())
    fwd_per_step = ra.times["forward_s"] / max(1, ra.times["forward_steps"])
    fwd_same = fwd_per_step * ra.adj
    # the direction of steepest ascent (the adjoint velocity cotangent on the fluid interior,
    # scaled to unit max-norm): the largest directional derivative, so the least FD noise
    fl = torch.as_tensor(np.ascontiguousarray(1.0 - pr.geom.iblank), device="cuda")
    inner = torch.zeros(pr.shape, dtype=torch.float64, device="cuda")
    inner[ra.sa.ops.I] = 1.0
    d = [c * fl * inner for c in cot[0]]
    scale = max(float(t.abs().max()) for t in d)
    d = [t / scale for t in d]
    adj_dot = sum(float((a * b).sum()) for a, b in zip(cot[0], d))
    h = 1e-3
    base = ra.checkpoints[ra.first]
    vals = []
    for sgn in (1.0, -1.0):
        st = dict(base)
        st["vel"] = [a + sgn * h * b for a, b in zip(base["vel"], d)]
        vals.append(float(loss_fn(ra.rerun(st, ra.adj))))
    fd = (vals[0] - vals[1]) / (2 * h)
    st = ra.sa.stats
    return {"loss": "mean u over the fluid cells of the cell plane nearest x = %g" % x_plane, "L": L,
            "adjoint_steps": ra.adj, "checkpoint_every": ra.every, "checkpoints": len(ra.checkpoints),
            "adjoint_s": ra.times["adjoint_s"], "recompute_s": ra.times["recompute_s"],
            "forward_s_same_steps": fwd_same, "adjoint_over_forward": ra.times["adjoint_s"] / fwd_same,
            "adjoint_peak_torch_bytes": adj_peak,
            "fd_check": {"h": h, "direction": "the adjoint's velocity cotangent at the first adjoint step on the "
                                             "fluid interior cells, scaled to unit max-norm", "fd": fd,
                         "adjoint": adj_dot,
                         "rel_diff": abs(fd - adj_dot) / max(abs(fd), 1e-300)},
            "left_null_s": ra.times.get("left_null_s"),
            "transposed_solves": {"momentum_gmres_applications": st.get("ad_transposed_applications", 0),
                                  "momentum_max_rel_residual": st.get("ad_transposed_rel_residual", 0.0),
                                  "momentum_s": st.get("ad_transposed_s", 0.0),
                                  "pressure_fgmres_applications": st.get("p_transposed_applications", 0),
                                  "pressure_max_rel_residual": st.get("p_transposed_rel_residual", 0.0),
                                  "pressure_s": st.get("p_transposed_s", 0.0),
                                  "rtol_momentum": ra.sa.rtol_ad, "rtol_pressure": ra.sa.rtol_p,
                                  "pressure_preconditioner": "one mixed-precision MG_Solver application",
                                  "warm_start": ra.sa.warm_start}}


def rel_l2_mean_free(pr, a, b):
    """Relative L2 distance (cell-volume weights, fluid cells) of two
    pressures after removing each one's volume-weighted fluid mean."""
    from flow_structure_interaction_fem_ibm_gb300.grid import Metrics
    n0, n1, n2 = pr.params.nx - 1, pr.params.ny - 1, pr.params.nz - 1
    I = (slice(1, n0 + 1), slice(1, n1 + 1), slice(1, n2 + 1))
    mx, my, mz = Metrics(pr.x), Metrics(pr.y), Metrics(pr.z)
    vol = mx.dx[1:n0 + 1, None, None] * my.dx[None, 1:n1 + 1, None] * mz.dx[None, None, 1:n2 + 1]
    w = vol * (1.0 - pr.geom.iblank[I])
    da = (a[I] - (a[I] * w).sum() / w.sum()) * (w > 0)
    db = (b[I] - (b[I] * w).sum() / w.sum()) * (w > 0)
    return float(np.sqrt(((da - db) ** 2 * vol).sum() / max((db ** 2 * vol).sum(), 1e-300)))


def config2_gpu(pr, solver_cls, krylov, reps=3):
    """Config 2 on the GPU: complete solves of the 128^3 stretched sphere at
    the config's tolerance in four forms (FP64 and mixed; the reference's
    stationary outer iteration and FGMRES(krylov)), each timed with CUDA
    events over `reps` solves after one warm-up, and an FP64 solve at 1e-4 of
    the tolerance as the converged reference."""
    import torch
    sh = pr.shape
    b = torch.from_numpy(np.ascontiguousarray(pr.nlu0.transpose(2, 1, 0))).cuda()
    p = torch.zeros(sh[::-1], dtype=torch.float64, device="cuda")
    out, fields = {}, {}
    forms = (("fp64_stationary", 0, 0), ("fp64_fgmres", 0, krylov), ("mixed_stationary", 1, 0),
             ("mixed_fgmres", 1, krylov), ("fp64_tight", 0, krylov))
    for name, mode, kr in forms:
        q = copy.deepcopy(pr.params)
        q.precision_mode, q.outer_krylov, q.iterMax_Poisson = mode, kr, 2000
        if name == "fp64_tight":
            # 1e-10: the compatibility shift holds the consistent part of the right-hand side
            # to about 1e-11 of max|nlu0|, so FP64 solves stall between 1e-11 and 1e-12
            q.restol_Poisson = pr.params.restol_Poisson * 1e-2
        s = solver_cls(q, pr.x, pr.y, pr.z).set_boundary(pr.geom)
        dev, iters, st = [], [], 0
        for r in range(1 + (reps if name != "fp64_tight" else 0)):
            p.zero_()
            torch.cuda.synchronize()
            st, it, mr, loc, d = s.solve_poisson_device(p.data_ptr(), b.data_ptr())
            if r > 0 or name == "fp64_tight":
                dev.append(d)
                iters.append(it)
        s.close()
        fields[name] = p.cpu().numpy().transpose(2, 1, 0).copy()
        out[name] = {"status": st, "iters": iters[-1], "seconds": float(np.median(dev)),
                     "solves_per_s": 1.0 / float(np.median(dev))}
    del b, p
    torch.cuda.empty_cache()
    return out, fields


def _section(fn, *a, **kw):
    """One auxiliary section of the benchmark line (projection steps, adjoint
    check, rollout): a failure is reported in the line as {"error": ...},
    with its traceback on stderr, instead of losing the measurements taken
    before it."""
    try:
        return fn(*a, **kw)
    except Exception as e:
        import traceback
        traceback.print_exc(file=sys.stderr)
        return {"error": f"{type(e).__name__}: {e}"}


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        return run_reference(args, rank, world)
    special = args.profile or args.profile_krylov or args.rollout > 0 or args.steps_only
    want_cpu = rank == 0 and world == 1 and not args.no_cpu_baseline and not special
    jobs = None
    if want_cpu:
        # CPU workers spawned before the first GPU call: one 256^3 outer iteration
        # of the oracle now, the complete 128^3 config-2 solve once its
        # right-hand side is ready
        jobs = OracleJobs(2)
        jobs.submit(1, "iteration", (args.n, args.seed))
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from flow_structure_interaction_fem_ibm_gb300.build import build_all
    if rank == 0:
        build_all()
    if world > 1:
        torch.distributed.barrier()
    from flow_structure_interaction_fem_ibm_gb300.poisson import PoissonSolver

    if args.profile_krylov:
        from flow_structure_interaction_fem_ibm_gb300 import problem as P
        pr = P.sphere(args.n, seed=args.seed, stretch=1.5)
        pp = copy.deepcopy(pr.params)
        pp.precision_mode, pp.outer_krylov, pp.iterMax_Poisson, pp.restol_Poisson = 1, args.krylov, 6, 0.0
        c = {"V": 1, "W": 2, "F": 3}[args.mgcycle]
        pp.mgcycle = (c, c, c)
        pp.iterFinest = args.iter_finest
        pp.omega = args.omega
        s = PoissonSolver(pp, pr.x, pr.y, pr.z).set_boundary(pr.geom)
        p = np.zeros(pr.shape, order="F")
        s.solve_poisson(p, pr.nlu0)
        print(json.dumps({"profile": "krylov", "stats": s.stats()}))
        s.close()
        return

    if args.rollout > 0:
        print(json.dumps(channel_rollout(args.rollout, args.rollout_cells, args.krylov,
                                         adjoint_steps=args.rollout_adjoint, iter_finest=args.iter_finest,
                                         omega=args.omega)))
        return

    if args.profile_fp64:
        from flow_structure_interaction_fem_ibm_gb300 import problem as P
        pr = P.sphere(args.n, seed=args.seed, stretch=1.5)
        s = PoissonSolver(pr.params, pr.x, pr.y, pr.z).set_boundary(pr.geom)   # plain FP64 handle
        sh = pr.shape[::-1]
        g = torch.Generator(device="cuda").manual_seed(1)
        rnd = lambda: torch.randn(sh, dtype=torch.float64, device="cuda", generator=g)
        u, v, w, pp = rnd(), rnd(), rnd(), rnd()
        faces = [torch.zeros(sh, dtype=torch.float64, device="cuda") for _ in range(3)]
        nlu0 = torch.zeros(sh, dtype=torch.float64, device="cuda")
        fp = [t.data_ptr() for t in faces]
        visc = torch.full(sh, 1e-3, dtype=torch.float64, device="cuda")
        nl = [torch.zeros(sh, dtype=torch.float64, device="cuda") for _ in range(3)]
        torch.cuda.synchronize()   # the library's stream does not wait for torch's
        s.face_vel_rhs(1e-3, u.data_ptr(), v.data_ptr(), w.data_ptr(), *fp, nlu0.data_ptr())
        s.correct_vel(1e-3, pp.data_ptr(), u.data_ptr(), v.data_ptr(), w.data_ptr(), *fp)
        s.rhs_advec_diff(1e-3, [u.data_ptr(), v.data_ptr(), w.data_ptr()], fp, visc.data_ptr(),
                         [t.data_ptr() for t in nl], advec_scheme=2)
        out = {k: s.time_kernel(w_, 0, 1) for k, w_ in (("calc_residual", 5), ("line_x_fp64", 0), ("dfma", 10))}
        torch.cuda.synchronize()
        print(json.dumps({"profile": "fp64", "grid": args.n, "ms_and_bytes": out}))
        s.close()
        return

    if args.steps_only:
        from flow_structure_interaction_fem_ibm_gb300 import problem as P
        pr = P.sphere(args.n, seed=args.seed, stretch=1.5)
        s = PoissonSolver(pr.params, pr.x, pr.y, pr.z).set_boundary(pr.geom)
        peaks = json.loads(PEAKS.read_text()) if PEAKS.exists() else {}
        out = projection_steps(s, pr, peaks.get("hbm_gbs", 6800.0))
        s.close()
        out["device_step"] = device_time_step(args.n, args.seed, args.tol, args.krylov)
        print(json.dumps({"profile": "projection_steps", "grid": args.n, "projection_steps": out}))
        return

    if args.profile:
        from flow_structure_interaction_fem_ibm_gb300 import problem as P
        pr = P.sphere(args.n, seed=args.seed, stretch=1.5)
        for mode in (1, 0):
            pp = copy.deepcopy(pr.params)
            pp.precision_mode, pp.iterMax_Poisson, pp.restol_Poisson = mode, 2, 0.0
            pp.omega = args.omega   # the headline's relaxation (the sweep kernels' relaxed store)
            s = PoissonSolver(pp, pr.x, pr.y, pr.z).set_boundary(pr.geom)
            p = np.zeros(pr.shape, order="F")
            s.solve_poisson(p, pr.nlu0)
            print(json.dumps({"profile": True, "precision_mode": mode, "stats": s.stats()}))
            s.close()
        return

    pr2 = shift2 = None
    if want_cpu:
        pr2, shift2 = config2_problem(args.tol, solver_cls=PoissonSolver)
        jobs.submit(0, "complete", (pr2.params, pr2.x, pr2.y, pr2.z, pr2.geom, pr2.nlu0))

    t_setup = time.perf_counter()
    pr, shift = build_problem(args.n, args.seed, args.tol, PoissonSolver)
    restol = pr.params.restol_Poisson

    cyc = {"V": 1, "W": 2, "F": 3}[args.mgcycle]

    def make(mode, krylov, **kw):
        q = copy.deepcopy(pr.params)
        q.precision_mode, q.outer_krylov = mode, krylov
        q.mgcycle = (cyc, cyc, cyc)
        q.iterFinest = args.iter_finest
        q.omega = args.omega
        for k, v in kw.items():
            setattr(q, k, v)
        return PoissonSolver(q, pr.x, pr.y, pr.z).set_boundary(pr.geom)

    s_mixed = make(1, args.krylov)
    s_fp64 = make(0, args.krylov)
    sh = pr.shape
    b = torch.from_numpy(np.ascontiguousarray(pr.nlu0.transpose(2, 1, 0))).cuda()
    p = torch.zeros(sh[::-1], dtype=torch.float64, device="cuda")
    setup_s = time.perf_counter() - t_setup

    def step(solver, must_converge=True):
        p.zero_()
        torch.cuda.current_stream().synchronize()
        st, it, mr, loc, dev_s = solver.solve_poisson_device(p.data_ptr(), b.data_ptr())
        if st != 0 and must_converge:
            raise RuntimeError(f"solve did not converge: status {st}, {it} iterations, maxres {mr}")
        return st, it, dev_s

    def timed(solver, k, w):
        for _ in range(w):
            step(solver)
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        l0 = solver.stats()["launches"]
        dev, iters = [], []
        t0 = time.perf_counter()
        for _ in range(k):
            _, it, d = step(solver)
            dev.append(d)
            iters.append(it)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        launches = solver.stats()["launches"] - l0
        tot = job_seconds(sum(dev), world)
        return tot, wall, iters, launches

    # headline: mixed precision, FGMRES(m) around the MG cycle (no instrumentation)
    with ClockSampler(local) as clk:
        mixed_s, mixed_wall, mixed_iters, mixed_launch = timed(s_mixed, args.steps, args.warmup)
        # the same timed steps again with CUDA events around every level-1 line
        # launch inside the solve graphs: the roofline's kernel durations
        s_mixed.line_timing(1)   # re-captures the graphs with the event records
        step(s_mixed)
        s_mixed.line_timing(1)   # reset the counters
        timed(s_mixed, args.steps, 0)
        lt = s_mixed.line_timing(0)["fp32"]
    clocks = clk.summary()
    value = replica_throughput(world, args.steps, mixed_s)

    k64 = max(2, args.steps // 2)
    fp64_s, fp64_wall, fp64_iters, _ = timed(s_fp64, k64, 1)
    fp64_value = replica_throughput(world, k64, fp64_s)

    # the reference's own stationary outer iteration (outer_krylov = 0), mixed: one full solve
    s_stat = make(1, 0, iterMax_Poisson=4000, mgcycle=(1, 1, 1), iterFinest=pr.params.iterFinest,
                  omega=pr.params.omega)
    st_stat, it_stat, dev_stat = step(s_stat, must_converge=False)
    s_stat.close()
    # FP64 stationary: time per outer iteration (the solve needs the same iteration count)
    s_stat64 = make(0, 0, iterMax_Poisson=12, restol_Poisson=0.0, mgcycle=(1, 1, 1),
                    iterFinest=pr.params.iterFinest, omega=pr.params.omega)
    step(s_stat64, must_converge=False)
    _, it64, dev64 = step(s_stat64, must_converge=False)
    s_stat64.close()
    # the headline forms with other cycles and smoothing counts (V-cycles with iterFinest 2
    # are the reference input's settings)
    cycles = {"headline": {"cycle": args.mgcycle, "iterFinest": args.iter_finest, "omega": args.omega}}
    for cname, fin, om, fname, mode in (("V", 2, 1.0, "mixed", 1), ("V", 1, 1.0, "mixed", 1),
                                        ("F", 2, 1.0, "mixed", 1), ("F", 1, 1.0, "mixed", 1),
                                        ("W", 2, 1.0, "mixed", 1), ("V", 2, 1.0, "fp64", 0),
                                        ("V", 1, 1.0, "fp64", 0)):
        c = {"V": 1, "W": 2, "F": 3}[cname]
        if c == cyc and fin == args.iter_finest and om == args.omega:
            continue
        sv = make(mode, args.krylov, mgcycle=(c, c, c), iterFinest=fin, omega=om)
        tc, _, itc, _ = timed(sv, 2, 1)
        cycles[f"{cname}_finest{fin}_omega{om:g}_{fname}"] = {"ms_per_solve": 1e3 * tc / 2, "iters": itc[0],
                                                              "solves_per_s": replica_throughput(world, 2, tc)}
        sv.close()
    stationary = {
        "cycle": "V, iterFinest as the reference input (the reference's own iteration)",
        "mixed": {"status": st_stat, "iters": it_stat, "seconds": dev_stat,
                  "solves_per_s": (1.0 / dev_stat) if st_stat == 0 else None},
        "fp64": {"ms_per_iteration": 1e3 * dev64 / it64,
                 "projected_seconds": dev64 / it64 * it_stat,
                 "note": "FP64 stationary solve = mixed stationary iteration count x measured FP64 time per iteration"},
    }

    # errors: mixed vs FP64 at the same tolerance, and vs an FP64 solve at restol/100
    fl = 1.0 - torch.from_numpy(np.ascontiguousarray(pr.geom.iblank.transpose(2, 1, 0))).cuda().double()
    n = args.n
    I = (slice(1, n + 1),) * 3

    def mean_free(t):
        a = t[I] * fl[I]
        return a - a.sum() / fl[I].sum() * fl[I]

    step(s_mixed)
    pm = mean_free(p.clone())
    step(s_fp64)
    pf = mean_free(p.clone())
    err = float(torch.linalg.vector_norm(pm - pf) / torch.linalg.vector_norm(pf))
    s_tight = make(0, args.krylov, restol_Poisson=restol * 1e-2, iterMax_Poisson=150)
    st_t, it_t, _ = step(s_tight, must_converge=False)
    s_tight.close()
    pt = mean_free(p.clone())
    err_tight = float(torch.linalg.vector_norm(pm - pt) / torch.linalg.vector_norm(pt))
    err64_tight = float(torch.linalg.vector_norm(pf - pt) / torch.linalg.vector_norm(pt))

    # config 3 at tolerance 1e-10: both forms timed, errors against an FP64 solve run to 1e-11
    # (the floor the compatibility shift leaves lies between 1e-11 and 1e-12)
    tol10 = {"tol": args.tol * 1e-2, "restol": restol * 1e-2}
    p10 = {}
    for name, mode in (("mixed", 1), ("fp64", 0)):
        sv = make(mode, args.krylov, restol_Poisson=restol * 1e-2, iterMax_Poisson=400)
        t10, _, it10, _ = timed(sv, 2, 1)
        p10[name] = mean_free(p.clone())
        tol10[name] = {"solves_per_s": replica_throughput(world, 2, t10), "ms_per_solve": 1e3 * t10 / 2,
                       "iters": it10[0]}
        sv.close()
    sv = make(0, args.krylov, restol_Poisson=restol * 1e-3, iterMax_Poisson=300)
    st12, it12, _ = step(sv, must_converge=False)
    sv.close()
    p12 = mean_free(p.clone())
    for name in ("mixed", "fp64"):
        tol10[name]["rel_l2_vs_fp64_1e11"] = float(torch.linalg.vector_norm(p10[name] - p12)
                                                   / torch.linalg.vector_norm(p12))
    tol10["mixed_over_fp64"] = tol10["mixed"]["solves_per_s"] / tol10["fp64"]["solves_per_s"]
    tol10["reference_solve"] = {"tol": args.tol * 1e-3, "status": st12, "iters": it12}
    del p10, p12

    # e2e through the host-buffer C ABI (fsi_mg_solve), pinned buffers
    e2e = None
    if not args.no_e2e:
        hp = torch.zeros(sh[::-1], dtype=torch.float64, pin_memory=True)
        hb = torch.from_numpy(np.ascontiguousarray(pr.nlu0.transpose(2, 1, 0))).pin_memory()
        hp_np = hp.numpy().transpose(2, 1, 0)
        hb_np = hb.numpy().transpose(2, 1, 0)
        hp_np[...] = 0.0
        s_mixed.solve_poisson(hp_np, hb_np)
        tot = 0.0
        k = max(2, args.steps // 2)
        for _ in range(k):
            hp_np[...] = 0.0
            st, it, mr, loc, _ = s_mixed.solve_poisson(hp_np, hb_np)
            if st != 0:
                raise RuntimeError(f"e2e solve did not converge: status {st}")
            tot += s_mixed.stats()["e2e_seconds"]
        # the library copies the (0:nx+1,0:ny+1,0:nz) part of each full array: the
        # (nz+1) plane is padding that no routine of the solve reads or writes
        nbytes = int(sh[0] * sh[1] * (sh[2] - 1)) * 8
        tot = job_seconds(tot, world)
        e2e = {"value": replica_throughput(world, k, tot), "unit": "solves/s", "h2d_bytes_per_step": 2 * nbytes,
               "d2h_bytes_per_step": nbytes}

    peaks = json.loads(PEAKS.read_text()) if PEAKS.exists() else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    steps_ops = None
    if not args.no_steps:
        steps_ops = _section(projection_steps, s_mixed, pr, peak)
        if "error" not in steps_ops:
            steps_ops["device_step"] = _section(device_time_step, args.n, args.seed, args.tol, args.krylov)

    # FP64 kernels against both roofs: HBM (measured copy bandwidth) and the FP64 pipe
    # (measured DFMA rate; FP64 thread-instructions per cell from the committed ncu summary)
    fp64_roofline = None
    if steps_ops is not None and "error" not in steps_ops:
        roof = steps_ops["fp64_roof"]["tflops"] * 1e12 / 2.0   # FP64-pipe thread-instructions per second
        ipc = profile_fp64_instr()
        cells = float(args.n) ** 3
        k = {"face_vel_rhs": steps_ops["no_van_kan"]["face_vel_rhs"],
             "correct_vel": steps_ops["no_van_kan"]["correct_vel"],
             "rhs_advec_diff": steps_ops["rhs_advec_diff_cn"]}
        ms_r, nb_r = s_fp64.time_kernel(5, 0, 20)
        k["calc_residual"] = {"device_us": 1e3 * ms_r, "alg_bytes": nb_r}
        ms_l, nb_l = s_fp64.time_kernel(0, 0, 20)
        k["line_fp64_x"] = {"device_us": 1e3 * ms_l, "alg_bytes": nb_l}
        fp64_roofline = {"fp64_roof_tflops": steps_ops["fp64_roof"]["tflops"], "hbm_peak_gbs": peak,
                         "instr_source": "profiles/fp64_kernels_160.md (ncu sm__inst_executed_pipe_fp64, not this run)",
                         "kernels": {}}
        for name, rec in k.items():
            t = rec["device_us"] * 1e-6
            ent = {"device_us": rec["device_us"], "hbm_frac": rec["alg_bytes"] / t / 1e9 / peak}
            if name in ipc:
                ent["fp64_pipe_frac"] = ipc[name] * cells / t / roof
            fp64_roofline["kernels"][name] = ent

    adjoint = None
    if rank == 0 and not args.no_adjoint:
        s_mixed.close()
        s_fp64.close()
        s_mixed = s_fp64 = None
        adjoint = _section(adjoint_check, args.adjoint_n, args.adjoint_dirs)

    rollout = None
    if rank == 0 and not args.no_rollout:
        # config 5: 200 steps; V-cycles: from the previous step's pressure a V-cycle FGMRES
        # reaches the tolerance in fewer, cheaper applications (111 ms per step against
        # 142 ms on F-cycles); the headline's relaxation: over 40 steps 17.1 instead of 20.2
        # applications per step and 97.8 instead of 108.8 ms per step at omega 1.5 vs 1
        rollout = _section(channel_rollout, 200, krylov=args.krylov, mgcycle=1, iter_finest=args.iter_finest,
                           omega=args.omega)

    # roofline of the dominant kernel: level-1 FP32 line relaxation (k_line_wp<float,dir,8>),
    # durations from CUDA events around each launch inside the timed solves
    avg_ms = lt["ms"] / max(lt["launches"], 1)
    achieved = lt["alg_bytes"] / (avg_ms * 1e-3) / 1e9
    traffic = profile_traffic(args.n)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic,
                "traffic_source": f"profiles/line_relaxation_fp32_{args.n}.md (ncu capture, not this run)",
                "kernel": "level-1 FP32 line relaxation, one colour per launch (x, y, z)",
                "launches": lt["launches"], "avg_us": 1e3 * avg_ms, "alg_bytes_per_launch": lt["alg_bytes"],
                "peak_source": "measured hbm_gbs" if PEAKS.exists() else "fallback"}

    cpu = config2 = model256 = None
    if want_cpu:
        # config 2 on the GPU while the oracle's complete solve runs on its core
        for sv in (s_mixed, s_fp64):
            if sv is not None:
                sv.close()
        s_mixed = s_fp64 = None
        g2, f2 = config2_gpu(pr2, PoissonSolver, args.krylov)
        ref2 = jobs.result(0, timeout=3600)
        it256 = jobs.result(1, timeout=3600)
        jobs.close()
        config2 = {"workload": "sphere_128^3_tanh1.5_r0.15_seed2_tol%g" % args.tol, "compat_shift": shift2,
                   "restol": pr2.params.restol_Poisson, "gpu": g2}
        if "error" not in ref2:
            t_ref = ref2["solve_s"]
            config2["oracle"] = {"status": ref2["status"], "iters": ref2["iters"], "maxres": ref2["maxres"],
                                 "seconds": t_ref, "solves_per_s": 1.0 / t_ref, "cores": 1,
                                 "host_cores": os.cpu_count(),
                                 "what": "complete solve_poisson of the oracle (serial C restatement of the "
                                         "reference MG, reference lexicographic line order), timed end to end"}
            po = ref2["p"]
            config2["parity"] = {
                "gpu_fp64_stationary_vs_oracle_rel_l2": rel_l2_mean_free(pr2, f2["fp64_stationary"], po),
                "gpu_fp64_fgmres_vs_oracle_rel_l2": rel_l2_mean_free(pr2, f2["fp64_fgmres"], po),
                "gpu_mixed_fgmres_vs_oracle_rel_l2": rel_l2_mean_free(pr2, f2["mixed_fgmres"], po),
                "oracle_vs_gpu_fp64_tight_rel_l2": rel_l2_mean_free(pr2, po, f2["fp64_tight"]),
                "gpu_fp64_stationary_vs_gpu_fp64_tight_rel_l2":
                    rel_l2_mean_free(pr2, f2["fp64_stationary"], f2["fp64_tight"]),
                "gpu_mixed_fgmres_vs_gpu_fp64_tight_rel_l2":
                    rel_l2_mean_free(pr2, f2["mixed_fgmres"], f2["fp64_tight"]),
                "note": "each solve stops inside its own residual ball at tol; the oracle's distance to the "
                        "tight solution (oracle_vs_gpu_fp64_tight) is the scale the GPU-vs-oracle figures "
                        "are read against"}
            config2["vs_reference"] = {k: g2[k]["solves_per_s"] * t_ref for k in
                                       ("fp64_stationary", "fp64_fgmres", "mixed_stationary", "mixed_fgmres")}
            cpu = {"value": 1.0 / t_ref, "unit": "solves/s", "cores": 1, "kind": "port",
                   "sample": ("one complete solve_poisson of the 128^3 config-2 workload (stretched sphere, "
                              f"tol {args.tol:g}; the 256^3 headline workload takes hours on one core) by the "
                              "oracle in the reference's line order, timed end to end on one of "
                              f"{os.cpu_count()} host cores; same run as the GPU's config2 solves")}
        else:
            config2["oracle"] = ref2
        if "error" not in it256:
            ref_it, src = REFERENCE_ITERATIONS[(args.n, args.seed, args.tol)] \
                if (args.n, args.seed, args.tol) in REFERENCE_ITERATIONS else (it_stat, "GPU stationary count")
            model256 = {"seconds_per_iteration": it256["seconds"], "iterations": ref_it, "iterations_source": src,
                        "solves_per_s": 1.0 / (it256["seconds"] * ref_it),
                        "what": (f"MODEL, not a timed solve: one oracle outer iteration at {args.n}^3 timed in "
                                 "this run x the reference's stationary iteration count")}

    out = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * mixed_s / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 cycle + f64 refinement", "data": "synthetic",
        "config": {"workload": f"sphere_{args.n}^3_tanh1.5_r0.15_tol{args.tol:g}_mixed_fgmres{args.krylov}",
                   "grid": args.n, "tol": args.tol, "restol": restol, "stretch": 1.5, "radius": 0.15,
                   "mg_cycle": args.mgcycle, "iterFinest": args.iter_finest, "omega": args.omega,
                   "triangles": 5120, "nGhost": int(pr.geom.nGhost), "compat_shift": shift,
                   "outer": f"FGMRES({args.krylov}) preconditioned by MG_Solver" if args.krylov else "stationary",
                   "l2": "inputs larger than L2 (two 139 MB FP64 fields + hierarchy)",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "fp64_value": fp64_value, "fp64_ms_per_step": 1e3 * fp64_s / k64,
        "mixed_over_fp64": value / fp64_value,
        "error": {"mixed_vs_fp64_rel_l2": err, "mixed_vs_fp64_tight_rel_l2": err_tight,
                  "fp64_vs_fp64_tight_rel_l2": err64_tight, "tight_restol": restol * 1e-2,
                  "tight_status": st_t, "tight_iters": it_t},
        "iters_mixed": mixed_iters[0], "iters_fp64": fp64_iters[0], "stationary": stationary, "cycles": cycles,
        "wall_ms_per_step": 1e3 * mixed_wall / args.steps,
        "gpu_launches": int(mixed_launch), "clocks": clocks, "e2e": e2e, "roofline": roofline,
        "cpu_baseline": cpu, "config2": config2, "reference_model_256": model256, "tol_1e10": tol10,
        "fp64_roofline": fp64_roofline,
        "adjoint": adjoint, "projection_steps": steps_ops, "channel_rollout": rollout,
        "setup_s": setup_s,
    }
    if rank == 0:
        print(json.dumps(out))
    for sv in (s_mixed, s_fp64):
        if sv is not None:
            sv.close()
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()

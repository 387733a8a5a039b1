"""Benchmark of the SHCI variational engine on one GB300 (or N replicas).

Workload (the largest of the synthetic workloads whose stated size fits one
GPU in the stored form): the synthetic molecular Hamiltonian with 24 spatial
orbitals, 12 alpha + 12 beta electrons, 72 Cholesky vectors (seeded), eps1
schedule 1e-3 -> 3e-4 -> 1e-4, one root. The whole variational stage runs in
the plain FP64 path (the reference's algorithm on the GPU), in the mixed
path with the reference's subspace, in the new form (mixed precision,
16-vector subspace, graph-captured iterations) with and without the learned
preconditioner, and in parity mode (loose and final Davidson tolerances both
1e-8, FP64 and new form). Each run's final determinant set is compared with
the FP64 run's (|dS| = size of the symmetric difference).

The timed "step" is one sigma (y = H x) over the final space of the FP64 run,
with the Hamiltonian resident in HBM. That space is the one the reference
algorithm selects (the oracle's FP64 run reproduces it determinant for
determinant), so the reference arm times its sigma on the same space.

value: sigma Mdets/s (N / t_sigma / 1e6), FP32 (mixed path), kernel-only,
device-resident vectors: two launches per step (shci_sigma_packed_device
gathers x into the stored matrix's storage order, then runs the sigma). e2e:
the same through the C-ABI call with pinned host buffers (shci_sigma: host->device
copy of x and device->host copy of y inside the timed region).

Further keys: `plain_fp64_sigma`, `block_k4_sigma`, `var` (the runs above),
`pt` (deterministic PT2 of the final space, eps2 1e-5, through
shci_pt_deterministic; `--section pt` times it alone), `rdm` (spatial 1- and
2-RDMs through shci_run_rdm), each with the CPU oracle on a bounded sample
beside it, and `configs` (the other synthetic workloads, including the
12-site Hubbard ring at its stated schedule, against the CPU oracle).
`--section sigma | direct | ham` times the stored sigmas, the matrix-free
sigma or the Hamiltonian build alone.

cpu_baseline: the oracle's restatement of the reference's rank-parallel
Hmult2 (rows dealt round-robin to one worker per host thread, private
accumulators summed) over the same final space, its lower triangle built by
the oracle from the GPU run's determinants.

--impl reference: Dice itself needs Boost and MPI, absent here, so the CPU
oracle (the reference's algorithm restated, threaded as the reference's MPI
ranks of one node would share the work) runs the same variational schedule
on the host cores, reproducing the FP64 final space, and its rank-parallel
sigma over that whole space is timed.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = "mol24"
WORKLOAD_DESC = ("mol24: synthetic molecular FCIDUMP n=24, 12a+12b, rank-72 Cholesky ERIs, seed "
                 "20260001, eps1 1e-3 -> 3e-4 -> 1e-4, 1 root; sigma over the final space of the FP64 "
                 "variational run")
# Davidson tolerance of parity mode (loose and final solves alike)
PARITY_TOL = 1e-8
# deterministic PT2 on the final mixed-precision space of the workload
PT_EPS2 = 1e-5
# DRAM bytes per mixed-sigma launch divided by its algorithmic bytes, from one
# ncu capture of the medium case (4.4983 GB measured read + write / 4.4633 GB
# algorithmic, profiles/sigma_mol24_medium.md); the full-size launch is too
# large to capture with all sections, and its traffic scales with the
# nonzeros it streams.
TRAFFIC_RATIO = 4.4983 / 4.4633


def dist_info():
    return (int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)),
            int(os.environ.get("LOCAL_RANK", 0)))


def replicas_throughput(t_local, units_per_rank, world, device="cpu"):
    """Whole-job throughput of `world` replicas: every rank processed
    units_per_rank units; the job took as long as its slowest rank (max over
    ranks of the local step time). Returns (units per second, max time)."""
    t = t_local
    if world > 1:
        import torch
        import torch.distributed as dist
        tt = torch.tensor([t_local], dtype=torch.float64, device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t = float(tt.item())
    return world * units_per_rank / t, t


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, gpu):
        self.path = tempfile.mktemp(suffix=".csv")
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(gpu), "--query-gpu=" + q, "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak_gbs():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return json.load(open(p))["hbm_gbs"], "measured"
    return 6800.0, "fallback"


def make_inputs(d, case="full", extra=()):
    """case "small": the same Hamiltonian stopped after two eps1 = 1e-3
    iterations (about 8e4 determinants, a ~0.8 GB Hamiltonian: larger than L2,
    small enough for a full ncu capture)."""
    from dice_gb300 import synthetic
    extra = tuple(synthetic.WORKLOADS[WORKLOAD].get("extra", ())) + tuple(extra)
    if case == "small":
        return synthetic.make_workload(WORKLOAD, d, schedule=[(0, 1e-3)], maxiter=2, extra=extra)
    if case == "medium":  # ~5.7e5 determinants: x no longer fits L1, a few GB on the device
        return synthetic.make_workload(WORKLOAD, d, schedule=[(0, 1e-3), (2, 3e-4)], maxiter=3, extra=extra)
    return synthetic.make_workload(WORKLOAD, d, extra=extra)


def sym_diff(a, b):
    """Size of the symmetric difference of two (N, 2) uint64 determinant lists."""
    va = np.ascontiguousarray(a, dtype=np.uint64).view(np.dtype((np.void, 16))).ravel()
    vb = np.ascontiguousarray(b, dtype=np.uint64).view(np.dtype((np.void, 16))).ravel()
    return int(len(np.setxor1d(va, vb)))


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def bench_config(world):
    """The `config` object both arms print (the same workload and space)."""
    return {"workload": WORKLOAD_DESC, "k_vectors": 1,
            "l2": "inputs larger than L2: the final-space Hamiltonian is tens of GB (5.4e9 nonzeros); no flush",
            "parallelism": "replicas" if world > 1 else "single GPU"}


def cpu_sigma_space(fcidump, dets, threads, seconds=10.0, max_reps=20):
    """The oracle's restatement of the reference's rank-parallel Hmult2 over the
    whole space `dets` (lower triangle built with `threads` workers; rows dealt
    round-robin to the workers, private full-length accumulators, summed),
    timed on the host cores for about `seconds`. Returns (lower-triangle
    entries, seconds per pass, passes)."""
    from oracle import oracle as orc
    orc.set_threads(threads)
    o = orc.Oracle(fcidump)
    nnz = o.ham_rows(dets, 1)
    x = np.random.default_rng(1).standard_normal(len(dets))
    o.sigma_mt(x, threads)  # warm-up
    times = []
    t_start = time.perf_counter()
    while len(times) < max_reps and (time.perf_counter() - t_start) < seconds:
        t0 = time.perf_counter()
        o.sigma_mt(x, threads)
        times.append(time.perf_counter() - t0)
    del o
    return nnz, statistics.mean(times), len(times)


def cpu_rdm_sample(fcidump, dets, stride=64):
    """The oracle holding every stride-th row of the space's lower triangle,
    for the RDM leg (a bounded sample; the oracle's RDM runs on one core).
    Returns (oracle, rows in the sample, entries)."""
    from oracle import oracle as orc
    o = orc.Oracle(fcidump)
    nnz = o.ham_rows(dets, stride)
    return o, (len(dets) + stride - 1) // stride, nnz


def run_reference(args):
    """The reference arm: the oracle (the reference's variational algorithm
    restated, with worker threads standing in for the MPI ranks of one node)
    runs the workload's whole FP64 variational schedule on the host cores,
    which reproduces the final space the GPU arm times, then times the
    reference's rank-parallel Hmult2 over that whole space."""
    rank, world, _ = dist_info()
    if rank != 0:
        return
    from oracle import oracle as orc
    orc.build()
    threads = host_threads()
    orc.set_threads(threads)
    with tempfile.TemporaryDirectory() as d:
        inp = make_inputs(d, args.case)
        t0 = time.perf_counter()
        run = orc.run_input(inp)
        t_var = time.perf_counter() - t0
        o = run.oracle
        n = len(run.dets)
        x = np.random.default_rng(1).standard_normal(n)
        for _ in range(args.warmup):
            o.sigma_mt(x, threads)
        times = []
        for _ in range(args.steps):
            t1 = time.perf_counter()
            o.sigma_mt(x, threads)
            times.append(time.perf_counter() - t1)
    t = statistics.mean(times)
    val = n / t / 1e6
    nnz_full = 2 * int(run.nnz_lower) - n
    sample = ("the whole final space (%d determinants, %d lower-triangle entries) of the oracle's FP64 run of the "
              "workload's schedule; the reference's rank-parallel Hmult2 (symmetric scatter in FP64, rows dealt "
              "round-robin to %d host threads standing in for its MPI ranks, private accumulators summed)"
              % (n, run.nnz_lower, threads))
    line = {"metric": "sigma Mdets/s (SHCI variational, stored H)", "value": val, "unit": "Mdets/s",
            "impl": "reference", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "config": bench_config(world),
            "space": {"n_dets": n, "nnz_offdiag": nnz_full - n, "nnz_lower": int(run.nnz_lower),
                      "ndets_per_iteration": [int(v) for v in run.ndets_log], "E_var": float(run.E[0])},
            "gnnz_s": nnz_full / t / 1e9,
            "var_wall_s": t_var,
            "cpu_baseline": {"value": val, "unit": "Mdets/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": val, "unit": "Mdets/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "Dice cannot be built here (needs Boost and MPI); the CPU oracle restating its variational "
                    "loop and rank-parallel sigma is run and timed"}
    print(json.dumps(line), flush=True)


def pt_section(e, E0, steps, cpu_leg, fcidump, eps2=PT_EPS2, warmup=1):
    """Deterministic PT2 (Epstein-Nesbet) of the final space through the
    C-ABI (host coefficients in, E2 out): candidates outside the variational
    space generated, merged and summed per second. CPU leg: the oracle's
    restatement on a bounded sample of parents (the middle of the space,
    doubled until it takes 5 s), against the whole space for removal."""
    ci = e.run_ci(1)[0]
    for _ in range(max(1, warmup)):
        e.pt_deterministic(ci, E0, eps2)  # warm-up: allocations
    import torch
    ts = []
    torch.cuda.nvtx.range_push("bench_pt")  # lets a profiler select exactly these launches
    for _ in range(max(2, steps // 4)):
        t0 = time.perf_counter()
        e2 = e.pt_deterministic(ci, E0, eps2)
        ts.append(time.perf_counter() - t0)
    torch.cuda.nvtx.range_pop()
    st = e.pt_stats()
    t = statistics.mean(ts)
    out = {"eps2": eps2, "ndets": len(ci), "E_var": E0, "E2": e2, "E_total": E0 + e2, "candidates": st["candidates"],
           "unique": st["unique"], "partitions": st["partitions"], "psi1_norm": st["psi1_norm"],
           "seconds": t, "reps": len(ts), "Mcand_s": st["candidates"] / t / 1e6,
           "what": "shci_pt_deterministic on the final mixed-precision space (the reference's "
                   "DoPerturbativeDeterministic): generation with atomic append, radix sort by "
                   "determinant, per-run exact numerator sums"}
    if cpu_leg:
        from oracle import oracle as orc
        dets = e.dets()
        o = orc.Oracle(fcidump)
        n = len(dets)
        p0, k = n // 2, 256
        while True:
            t0 = time.perf_counter()
            _, sto = o.pt_det_range(dets, ci, E0, eps2, p0, min(n, p0 + k))
            tc = time.perf_counter() - t0
            if tc > 5.0 or p0 + k >= n:
                break
            k *= 2
        out["cpu_oracle"] = {"Mcand_s": sto["outside"] / tc / 1e6, "cores": 1, "kind": "port", "seconds": tc,
                             "sample": "parents [%d, %d) of %d, %d candidates outside the space"
                                       % (p0, min(n, p0 + k), n, sto["outside"])}
        out["speedup_vs_cpu_oracle"] = out["Mcand_s"] / out["cpu_oracle"]["Mcand_s"]
    return out


def rdm_section(e, nnz_offdiag, cpu):
    """Spatial 1- and 2-RDMs of root 0 on the final space through the C-ABI
    (shci_run_rdm, results copied to the host): connected pairs J < I per
    second. CPU leg: the oracle's restatement of EvaluateRDM + EvaluateOneRDM
    on its stored connection lists of the sigma sample."""
    import torch
    e.rdm()  # warm-up
    ts = []
    torch.cuda.nvtx.range_push("bench_rdm")
    for _ in range(3):
        t0 = time.perf_counter()
        s2, s1 = e.rdm()
        ts.append(time.perf_counter() - t0)
    torch.cuda.nvtx.range_pop()
    t = statistics.mean(ts)
    conn = nnz_offdiag // 2
    out = {"what": "shci_run_rdm on the final mixed-precision space (the reference's EvaluateRDM + "
                   "EvaluateOneRDM): fixed-point integer atomics over the stored connection lists",
           "n_dets": e.ndets(), "connections": conn, "seconds": t, "Gconn_s": conn / t / 1e9,
           "trace_1rdm": float(np.trace(s1))}
    if cpu is not None:
        o, n, rows, nnz_lower = cpu
        x = np.random.default_rng(3).standard_normal(n)
        x /= np.linalg.norm(x)
        t0 = time.perf_counter()
        o.rdm_on_ham(x)
        tc = time.perf_counter() - t0
        out["cpu_oracle"] = {"Gconn_s": (nnz_lower - rows) / tc / 1e9, "cores": 1, "kind": "port", "seconds": tc,
                             "sample": "every 64-th row of the same final space (%d rows), %d connected pairs"
                                       % (rows, nnz_lower - rows)}
        out["speedup_vs_cpu_oracle"] = out["Gconn_s"] / out["cpu_oracle"]["Gconn_s"]
    return out


def run_pt_only(args):
    """--section pt: the variational stage in the mixed path on the chosen
    case, then the perturbative stage timed alone (one JSON line)."""
    import torch
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    from dice_gb300 import engine as eng
    work = tempfile.mkdtemp()
    inp = make_inputs(work, args.case)
    e = eng.Engine(local)
    E = e.run_input(inp, mode="mixed")
    l0 = e.launch_count()
    pt = pt_section(e, float(E[0]), args.steps, rank == 0 and not args.no_cpu, os.path.join(work, "FCIDUMP"),
                    eps2=args.pt_eps2, warmup=args.warmup)
    launches = (e.launch_count() - l0) // (pt["reps"] + args.warmup)
    e.close()
    line = {"metric": "PT2 candidates/s (deterministic Epstein-Nesbet)", "value": pt["Mcand_s"],
            "unit": "Mcand/s", "n_gpus": 1, "steps": pt["reps"], "warmup": args.warmup,
            "ms_per_step": pt["seconds"] * 1e3, "higher_is_better": True, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "mol24 (%s case): %d determinants, eps2 %g" % (args.case, pt["ndets"], pt["eps2"])},
            "gpu_launches": launches, "pt": pt}
    if rank == 0:
        print(json.dumps(line), flush=True)


def other_configs(work, device):
    """The other workloads: the 12-site Hubbard ring at its stated schedule
    against the oracle, and the mol36, mol64 and mol50 generators at the
    sizes a bench run affords, each the plain FP64 GPU path against the new
    form on the same input (final Davidson solve to 1e-6, loose solves at the
    reference's 5e-5): mol36 with 4 roots in block Davidson, mol64
    matrix-free with 4 roots, mol50 with and without the learned
    preconditioner."""
    from dice_gb300 import engine as eng, synthetic

    def run(name, sched, maxiter, mode, block, precond="plain", basis=(0, 0), extra=()):
        inp = synthetic.make_workload(name, os.path.join(work, name), schedule=sched, maxiter=maxiter,
                                      extra=("davidsonTol 1e-6",) + tuple(extra))
        g = eng.Engine(device)
        g.set_preconditioner(precond)
        g.set_davidson_basis(*basis)
        E = g.run_input(inp, mode=mode, block=block)
        t, st, lg = g.timings(), g.run_stats(), g.run_log()
        dets = g.dets()
        g.close()
        return {"E_var": [float(v) for v in E], "wall_s": t["total"], "ham_s": t["ham"], "davidson_s": t["davidson"],
                "sigma_s": t["sigma"], "davidson_iters": int(st["davidson_iters"]),
                "ndets": [int(v) for v in lg["ndets"]], "_dets": dets}

    out = {}
    # the 12-site Hubbard ring at its stated schedule, GPU paths
    # against the oracle's serial run on one host core
    from oracle import oracle as orc
    hub = synthetic.make_workload("hubbard12", os.path.join(work, "hubbard12"))
    orc.set_threads(1)
    t0 = time.perf_counter()
    oref = orc.run_input(hub)
    t_orc = time.perf_counter() - t0
    res = {}
    for key, mode, basis in (("fp64", "fp64", (0, 0)), ("new_form", "mixed", (16, 8))):
        g = eng.Engine(device)
        g.set_davidson_basis(*basis)
        E = g.run_input(hub, mode=mode)
        t = g.timings()
        res[key] = {"E_var": float(E[0]), "wall_s": t["total"], "ndets": [int(v) for v in g.run_log()["ndets"]],
                    "dS_vs_oracle": sym_diff(g.dets(), oref.dets), "dE_vs_oracle": float(E[0] - oref.E[0])}
        g.close()
    out["hubbard12_stated_schedule"] = {
        "what": "1-D Hubbard ring, 12 sites, t=1, U=4, 6a+6b, eps1 1e-3 (x3) then 1e-4, maxiter 6, 1 root, "
                "stated schedule; GPU FP64 and new form against the oracle's FP64 run",
        "oracle": {"E_var": float(oref.E[0]), "wall_s": t_orc, "ndets": [int(v) for v in oref.ndets_log],
                   "cores": 1, "kind": "port"},
        **res, "fp64_speedup_vs_oracle": t_orc / res["fp64"]["wall_s"]}
    # mol36 (n=36, 14a+14b, 4 roots, block Davidson): eps1
    # 1e-3 twice then 6e-4 (eps1 3e-4 already selects 5.8 M determinants,
    # whose stored matrix does not fit beside the FP64 run's)
    # in parity mode (loose solves as tight as the final one), so that both
    # paths select the same determinants and the roots compare one to one
    sched = [(0, 1e-3), (2, 6e-4)]
    par = ("davidsonTolLoose 1e-6",)
    ref = run("mol36", sched, 3, "fp64", True, extra=par)
    new = run("mol36", sched, 3, "mixed", True, basis=(16, 12), extra=par)
    out["mol36_4roots_block"] = {
        "what": "mol36: n=36, 14a+14b, 4 roots, block Davidson (k=4 per sigma launch), eps1 "
                "1e-3 x2 -> 6e-4, parity mode (every solve to 1e-6) (eps1 3e-5 selects far more determinants than "
                "one GPU holds in the stored form)",
        "fp64": ref, "new_form": new, "dE_per_root": [a - b for a, b in zip(new["E_var"], ref["E_var"])],
        "dS": sym_diff(new.pop("_dets"), ref.pop("_dets")), "wall_speedup": ref["wall_s"] / new["wall_s"]}
    # mol64 (n=64, 20a+20b, two-word determinants), 4 roots,
    # matrix-free: eps1 2e-3 twice
    # one selection (the same space for both paths: the reference forces the
    # loose tolerance of matrix-free runs to 3e-2, SHCI/input.cpp, so later
    # selections differ), then two for scale
    for key, sched, it in (("mol64_4roots_matrix_free", [(0, 1e-3)], 1),
                           ("mol64_4roots_matrix_free_2iter", [(0, 2e-3)], 2)):
        ref = run("mol64", sched, it, "fp64", True, extra=("DirectDavidson",))
        new = run("mol64", sched, it, "mixed", True, extra=("DirectDavidson",))
        out[key] = {
            "what": "mol64: n=64, 20a+20b (two-word determinants), 4 roots, matrix-free sigma, "
                    "schedule %s" % sched,
            "fp64": ref, "mixed": new, "dE_per_root": [a - b for a, b in zip(new["E_var"], ref["E_var"])],
            "dS": sym_diff(new.pop("_dets"), ref.pop("_dets")), "wall_speedup": ref["wall_s"] / new["wall_s"]}
    # mol50 (n=50, 16a+16b): eps1 1e-3 twice then 3e-4 (2.3 M
    # determinants), learned preconditioner against the plain one
    sched = [(0, 1e-3), (2, 3e-4)]
    plain = run("mol50", sched, 3, "mixed", False, "plain")
    mlp = run("mol50", sched, 3, "mixed", False, "mlp")
    dS50 = sym_diff(plain.pop("_dets"), mlp.pop("_dets"))
    out["mol50_learned_preconditioner"] = {
        "what": "mol50: n=50, 16a+16b, 1 root, mixed precision, reference subspace, eps1 1e-3 x2 "
                "-> 3e-4; learned preconditioner (trained on Davidson's residual/correction pairs, judged by the "
                "plain one) against the plain diagonal preconditioner",
        "plain": plain, "mlp": mlp, "dE": mlp["E_var"][0] - plain["E_var"][0], "dS": dS50,
        "wall_speedup_mlp_vs_plain": plain["wall_s"] / mlp["wall_s"]}
    return out


def run_ours(args):
    import torch
    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    from dice_gb300 import engine as eng

    work = tempfile.mkdtemp()
    inp = make_inputs(work, args.case)
    inp_parity = make_inputs(os.path.join(work, "parity"), args.case,
                             extra=("davidsonTol %g" % PARITY_TOL, "davidsonTolLoose %g" % PARITY_TOL))
    e = eng.Engine(local)

    # the whole variational stage, six ways; the plain FP64 run (the
    # reference's algorithm) comes last, so that its final space, the one the
    # reference arm reproduces, stays resident for the sigma steps below
    def var_run(what, path, mode, precond, basis):
        e.set_preconditioner(precond)
        e.set_davidson_basis(*basis)
        E = e.run_input(path, mode=mode)
        t, st, lg = e.timings(), e.run_stats(), e.run_log()
        return {"E_var": float(E[0]), "wall_s": t["total"], "stages_s": t, "what": what,
                "davidson_iters_total": int(st["davidson_iters"]), "mlp_train_s": st["t_mlp"],
                "ndets": [int(v) for v in lg["ndets"]], "davidson_iters": [int(v) for v in lg["davidson"]],
                "_dets": e.dets()}

    NF = "mixed precision (FP32 sigma, float-float refinement) + 16-vector Davidson subspace collapsed to 8, " \
         "graph-captured iterations"
    runs = {
        "new_form": var_run(NF, inp, "mixed", "plain", (16, 8)),
        "new_form_mlp": var_run("new form + learned (BF16 MLP) preconditioner trained during the run", inp, "mixed",
                                "mlp", (16, 8)),
        "mixed": var_run("mixed precision with the reference's Davidson subspace", inp, "mixed", "plain", (0, 0)),
        "parity_fp64": var_run("parity mode, plain FP64 path: loose and final Davidson tolerance %g" % PARITY_TOL,
                               inp_parity, "fp64", "plain", (0, 0)),
        "parity_new_form": var_run("parity mode, new form: loose and final Davidson tolerance %g" % PARITY_TOL,
                                   inp_parity, "mixed", "plain", (16, 8)),
        "fp64": var_run("plain FP64 GPU path: the reference's algorithm", inp, "fp64", "plain", (0, 0)),
    }
    N = e.ndets()
    dets_fp64 = runs["fp64"]["_dets"]
    ref64 = runs["fp64"]
    for key, r in runs.items():
        if key.startswith("parity"):
            continue
        r["dS_vs_fp64"] = sym_diff(r["_dets"], dets_fp64)
        r["dE_vs_fp64"] = r["E_var"] - ref64["E_var"]
        r["wall_speedup_vs_fp64"] = ref64["wall_s"] / r["wall_s"]
    var = {k: {kk: vv for kk, vv in r.items() if not kk.startswith("_")} for k, r in runs.items()}
    var["parity_mode"] = {
        "dS_new_form_vs_fp64": sym_diff(runs["parity_new_form"]["_dets"], runs["parity_fp64"]["_dets"]),
        "dE_new_form_minus_fp64": runs["parity_new_form"]["E_var"] - runs["parity_fp64"]["E_var"],
        "dS_parity_fp64_vs_default_fp64": sym_diff(runs["parity_fp64"]["_dets"], dets_fp64),
        "wall_speedup_new_form_vs_fp64": runs["parity_fp64"]["wall_s"] / runs["parity_new_form"]["wall_s"]}
    del runs

    stream = torch.cuda.ExternalStream(e.stream, device=torch.device("cuda", local))
    k = 1
    rng = np.random.default_rng(5)
    x_host = rng.standard_normal(N)

    def timed_sigma(mode, packed, nsteps, nwarm, kp=1):
        nnz = e.ham_build(mode)
        y = torch.zeros(kp * N, dtype=torch.float64, device="cuda")
        for _ in range(nwarm):
            e.sigma_packed_device(packed.data_ptr(), kp, kp, y.data_ptr(), N, mode=mode)
        torch.cuda.synchronize()
        csr_bytes, _ = e.ham_bytes()
        flush = None
        if csr_bytes < 2 * 129 * 2 ** 20:
            flush = torch.empty(256 * 2 ** 20 // 4, dtype=torch.float32, device="cuda")
        ts = []
        l0 = e.launch_count()
        # NVTX range so that a profiler can select exactly these launches
        torch.cuda.nvtx.range_push("bench_sigma_%s_k%d" % (mode, kp))
        for _ in range(nsteps):
            if flush is not None:
                with torch.cuda.stream(stream):
                    flush.fill_(1.0)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            e.sigma_packed_device(packed.data_ptr(), kp, kp, y.data_ptr(), N, mode=mode)
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b) * 1e-3)
        torch.cuda.nvtx.range_pop()
        launches = e.launch_count() - l0
        return nnz, ts, launches, flush is not None, y, e.sigma_bytes(mode, kp)

    x_dev = torch.tensor(x_host, device="cuda")
    # plain FP64 sigma on the FP64 run's matrix
    nnz64, ts64, _, _, y64, alg64 = timed_sigma("fp64", x_dev, max(3, args.steps // 2), args.warmup)
    # mixed FP32 sigma (the timed region of `value`) on the same space
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = Clocks(local)
    wall0 = time.perf_counter()
    nnz, ts32, launches, flushed, y32, alg_bytes = timed_sigma("mixed", x_dev.float(), args.steps, args.warmup)
    wall = time.perf_counter() - wall0
    clk = clocks.stop()
    torch.cuda.synchronize()
    rate, t_max = replicas_throughput(statistics.mean(ts32), k * N, world, device="cuda")
    value = rate / 1e6
    sig_err = float((y32 - y64).abs().max() / y64.abs().max())
    # block sigma: k = 4 vectors per pass (the block-Davidson launch)
    x4 = torch.tensor(rng.standard_normal((N, 4)), device="cuda").float().contiguous()
    _, ts4, _, _, _, alg4 = timed_sigma("mixed", x4, max(3, args.steps // 2), args.warmup, kp=4)
    t4 = statistics.mean(ts4)

    # end to end through the C-ABI (shci_sigma) with pinned host buffers: each
    # step copies x to the device and y back inside the call
    x_pin = torch.tensor(np.ascontiguousarray(x_host, dtype=np.float64).reshape(k, N)).pin_memory()
    y_pin = torch.empty((k, N), dtype=torch.float64).pin_memory()
    for _ in range(2):
        e.sigma_host(x_pin.data_ptr(), y_pin.data_ptr(), k, "mixed")
    te = []
    for _ in range(max(3, args.steps // 2)):
        t0 = time.perf_counter()
        e.sigma_host(x_pin.data_ptr(), y_pin.data_ptr(), k, "mixed")
        te.append(time.perf_counter() - t0)
    e2e = world * k * N / statistics.mean(te) / 1e6

    peak, peak_kind = measured_peak_gbs()
    # algorithmic bytes of each launch as the library lays the matrix out
    # (k = 1 mixed: 16-bit column deltas + FP32 values, 6 B per stored entry)
    achieved = alg_bytes / t_max / 1e9
    ach64 = alg64 / statistics.mean(ts64) / 1e9

    cpu = None
    cpu_rdm = None
    fcidump = os.path.join(os.path.dirname(inp), "FCIDUMP")
    if rank == 0 and not args.no_cpu:
        from oracle import oracle as orc
        orc.build()
        threads = host_threads()
        nnz_l, tc, reps = cpu_sigma_space(fcidump, dets_fp64, threads)
        cpu = {"value": N / tc / 1e6, "unit": "Mdets/s", "cores": threads, "kind": "port",
               "sample": "the same final space (%d determinants, %d lower-triangle entries built by the oracle); "
                         "the oracle's restatement of the reference's rank-parallel Hmult2 (FP64 symmetric scatter, "
                         "%d host threads as its MPI ranks, private full-length accumulators summed), %d passes"
                         % (N, nnz_l, threads, reps)}
        o, rows, nnz_rows = cpu_rdm_sample(fcidump, dets_fp64)
        cpu_rdm = (o, N, rows, nnz_rows)

    line = {
        "metric": "sigma Mdets/s (SHCI variational, stored H)", "value": value, "unit": "Mdets/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64 diagonal, FP64 refinement)",
        "data": "synthetic",
        "config": bench_config(world),
        "space": {"n_dets": N, "nnz_offdiag": nnz, "ndets_per_iteration": var["fp64"]["ndets"],
                  "E_var": var["fp64"]["E_var"]},
        "gnnz_s": (nnz + N) / t_max / 1e9,
        "e2e": {"value": e2e, "unit": "Mdets/s", "h2d_bytes_per_step": N * k * 8, "d2h_bytes_per_step": N * k * 8,
                "host_buffers": "pinned"},
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": alg_bytes * TRAFFIC_RATIO, "traffic_note": "scaled from the medium-case ncu capture",
                     "peak_kind": peak_kind, "alg_bytes_per_launch": alg_bytes},
        "plain_fp64_sigma": {"mdets_s": k * N / statistics.mean(ts64) / 1e6, "achieved_gbs": ach64,
                             "frac": ach64 / peak, "nnz": nnz64},
        "mixed_vs_fp64_sigma_speedup": statistics.mean(ts64) / t_max,
        "block_k4_sigma": {"mdets_s": 4 * N / t4 / 1e6, "ms": t4 * 1e3, "achieved_gbs": alg4 / t4 / 1e9,
                           "frac": alg4 / t4 / 1e9 / peak},
        "sigma_rel_err_fp32_vs_fp64": sig_err,
        "var": var,
        "clocks": clk, "timed_wall_s": wall,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    line["pt"] = pt_section(e, var["fp64"]["E_var"], args.steps, rank == 0 and not args.no_cpu, fcidump)
    line["rdm"] = rdm_section(e, nnz, cpu_rdm)
    e.close()
    if args.case == "full" and not args.no_configs:
        line["configs"] = other_configs(work, local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def run_sigma_only(args):
    """--section sigma: the plain FP64 variational run of the chosen case, then
    the stored sigmas timed alone on its final space (FP64 k = 1, mixed k = 4,
    mixed k = 1), one JSON line. Each kind of launch runs inside its own NVTX
    range (bench_sigma_<mode>_k<k>), so a profiler can select exactly it."""
    import torch
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    from dice_gb300 import engine as eng
    work = tempfile.mkdtemp()
    inp = make_inputs(work, args.case)
    e = eng.Engine(local)
    e.run_input(inp, mode="fp64")
    N = e.ndets()
    stream = torch.cuda.ExternalStream(e.stream, device=torch.device("cuda", local))
    rng = np.random.default_rng(5)
    out = {"case": args.case, "n_dets": N}
    peak, _ = measured_peak_gbs()
    for mode, kp in (("fp64", 1), ("mixed", 4), ("mixed", 1)):
        nnz = e.ham_build(mode)
        x = torch.tensor(rng.standard_normal((N, kp)), device="cuda")
        if mode == "mixed":
            x = x.float()
        x = x.contiguous()
        y = torch.zeros(kp * N, dtype=torch.float64, device="cuda")
        for _ in range(args.warmup):
            e.sigma_packed_device(x.data_ptr(), kp, kp, y.data_ptr(), N, mode=mode)
        torch.cuda.synchronize()
        ts = []
        torch.cuda.nvtx.range_push("bench_sigma_%s_k%d" % (mode, kp))
        for _ in range(args.steps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            e.sigma_packed_device(x.data_ptr(), kp, kp, y.data_ptr(), N, mode=mode)
            b.record(stream)
            b.synchronize()
            ts.append(a.elapsed_time(b) * 1e-3)
        torch.cuda.nvtx.range_pop()
        t = statistics.median(ts)
        alg = e.sigma_bytes(mode, kp)
        out["%s_k%d" % (mode, kp)] = {"ms": t * 1e3, "mdets_s": kp * N / t / 1e6, "nnz": nnz, "alg_bytes": alg,
                                      "achieved_gbs": alg / t / 1e9, "frac": alg / t / 1e9 / peak}
    e.close()
    if rank == 0:
        print(json.dumps(out), flush=True)


def run_ham_only(args):
    """--section ham: the plain FP64 variational run of the chosen case, then
    the Hamiltonian of its final space built from scratch (string tables,
    partial-string index, diagonal, count, emit, row sort; for the mixed form
    also the 16-bit-delta copy), FP64 and mixed, each timed build inside its
    own NVTX range (bench_ham_<mode>). Reloading the determinants before each
    build drops every table and the stored matrix."""
    import torch
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    from dice_gb300 import engine as eng
    work = tempfile.mkdtemp()
    inp = make_inputs(work, args.case)
    e = eng.Engine(local)
    e.run_input(inp, mode="fp64")
    dets = e.dets()
    out = {"case": args.case, "n_dets": len(dets)}
    for mode in ("fp64", "mixed"):
        ts = []
        nnz = 0
        for it in range(args.warmup + args.steps):
            e.set_dets(dets)
            torch.cuda.synchronize()
            timed = it >= args.warmup
            if timed:
                torch.cuda.nvtx.range_push("bench_ham_" + mode)
            t0 = time.perf_counter()
            nnz = e.ham_build(mode)
            torch.cuda.synchronize()
            if timed:
                ts.append(time.perf_counter() - t0)
                torch.cuda.nvtx.range_pop()
        t = statistics.median(ts)
        out[mode] = {"s": t, "nnz": nnz, "gnnz_s": nnz / t / 1e9}
    e.close()
    if rank == 0:
        print(json.dumps(out), flush=True)


def run_large(args):
    """--section large: the mol36 workload (n=36, 14a+14b, 4 roots, block
    Davidson) at millions of determinants (5.8 M at eps1 3e-4; 2e-4 selects
    24.6 M), run with the matrix-free sigma in FP64 (the reference's
    DirectDavidson path): eps1 1e-3 twice, then 3e-4, final solve to 1e-6.
    Prints the determinant counts, per-root energies, stage times and the
    sigma throughput. Takes minutes."""
    import torch
    from dice_gb300 import engine as eng, synthetic
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    work = tempfile.mkdtemp()
    inp = synthetic.make_workload("mol36", work, schedule=[(0, 1e-3), (2, 3e-4)], maxiter=3,
                                  extra=("davidsonTol 1e-6", "DirectDavidson"))
    e = eng.Engine(local)
    t0 = time.perf_counter()
    E = e.run_input(inp, mode="fp64", block=True)
    wall = time.perf_counter() - t0
    t, st, lg = e.timings(), e.run_stats(), e.run_log()
    N = e.ndets()
    x = np.random.default_rng(2).standard_normal((4, N))
    e.sigma(x, "direct")
    ts = []
    for _ in range(2):
        a = time.perf_counter()
        e.sigma(x, "direct")
        ts.append(time.perf_counter() - a)
    e.close()
    out = {"workload": "mol36 (n=36, 14a+14b, rank-108 ERIs), 4 roots, block Davidson, matrix-free FP64 sigma, "
                       "eps1 1e-3 x2 -> 3e-4, final solve 1e-6",
           "n_dets": N, "ndets": [int(v) for v in lg["ndets"]], "E_var": [float(v) for v in E], "wall_s": wall,
           "stages_s": t, "davidson_iters": int(st["davidson_iters"]), "sigma_k4_s": statistics.median(ts),
           "mdets_s": 4 * N / statistics.median(ts) / 1e6}
    if rank == 0:
        print(json.dumps(out), flush=True)


def run_direct_only(args):
    """--section direct: the matrix-free sigma timed alone. The space is the
    mol36 workload's (n=36, 14a+14b, rank-108 ERIs, seed 20260002) after
    two eps1 = 1e-3 iterations of a stored FP64 run with four roots (about
    5e5 determinants); then four-vector FP32 and FP64 matrix-free sigmas, each
    inside its own NVTX range (bench_direct_<mode>), with the stored matrix's
    nonzero count as the element count."""
    import torch
    from dice_gb300 import engine as eng, synthetic
    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    work = tempfile.mkdtemp()
    inp = synthetic.make_workload("mol36", work, schedule=[(0, 1e-3)], maxiter=2)
    e = eng.Engine(local)
    e.run_input(inp, mode="fp64", block=True)
    N = e.ndets()
    nnz = e.ham_build("fp64")
    x = np.random.default_rng(1).standard_normal((4, N))
    out = {"workload": "mol36 (n=36, 14a+14b, rank-108 ERIs), eps1 1e-3 x2", "n_dets": N, "nnz_offdiag": nnz, "k": 4}
    for mode in ("direct_mixed", "direct"):
        e.ham_build(mode)
        for _ in range(args.warmup):
            e.sigma(x, mode)
        ts = []
        torch.cuda.nvtx.range_push("bench_direct_" + mode)
        for _ in range(args.steps):
            t0 = time.perf_counter()
            e.sigma(x, mode)
            ts.append(time.perf_counter() - t0)
        torch.cuda.nvtx.range_pop()
        t = statistics.median(ts)
        out[mode] = {"s": t, "gelem_s": nnz / t / 1e9, "mdets_s": 4 * N / t / 1e6}
    e.close()
    if rank == 0:
        print(json.dumps(out), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-configs", action="store_true", help="skip the other workloads (mol36, mol64, mol50)")
    ap.add_argument("--case", default="full", choices=["full", "medium", "small"],
                    help="small: the profiling case (two eps1 = 1e-3 iterations)")
    ap.add_argument("--section", default="all", choices=["all", "pt", "sigma", "direct", "ham", "large"],
                    help="pt: only the variational run and the timed perturbative stage; sigma: only the FP64 run "
                         "and the stored sigmas (FP64 k=1, mixed k=4, mixed k=1) timed on its space; direct: the "
                         "matrix-free sigma (k=4, FP32 and FP64) on mol36 (n=36, 14a+14b); ham: the FP64 run, "
                         "then its Hamiltonian built from scratch (FP64 and mixed); large: mol36 with 4 roots at 5.8 M "
                         "determinants, matrix-free (minutes)")
    ap.add_argument("--pt-eps2", type=float, default=PT_EPS2)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.section == "pt":
        run_pt_only(args)
    elif args.section == "sigma":
        run_sigma_only(args)
    elif args.section == "ham":
        run_ham_only(args)
    elif args.section == "large":
        run_large(args)
    elif args.section == "direct":
        run_direct_only(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

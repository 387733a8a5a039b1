"""Benchmark of the SHCI variational engine on one GB300 (or N replicas).

Workload: the synthetic molecular Hamiltonian with 24 spatial orbitals,
12 alpha + 12 beta electrons, 72 Cholesky vectors (seeded), eps1 schedule
1e-3 -> 3e-4 -> 1e-4, one root. The whole variational stage is run in the
mixed path (FP32 sigma + FP64 refinement) and in the plain FP64 path; the
timed "step" is then one sigma (y = H x) over the final variational space
with the Hamiltonian resident in HBM.

value: sigma Mdets/s (N / t_sigma / 1e6), kernel-only, device-resident
vectors: two launches per step (shci_sigma_packed_device gathers x into the
stored matrix's storage order, then runs the sigma). e2e: the same through the C-ABI call with host buffers
(shci_sigma: host->device copy of x and device->host copy of y inside the
timed region). Extra keys report the variational wall time and E_var of
both paths.

Further keys: `pt` (deterministic PT2 of the final space, eps2 1e-5, through
shci_pt_deterministic; `--section pt` times it alone), `rdm` (spatial 1- and
2-RDMs of the final space through shci_run_rdm), each with the CPU oracle on a
bounded sample beside it, and `configs` (the other synthetic workloads).

--impl reference: the CPU oracle's restatement of Dice's sigma (Dice itself
needs Boost and MPI, absent here) timed on a bounded sample of the same
workload, in the reference's rank-parallel form (rows dealt round-robin to
one worker per host thread, as Dice's MPI ranks on one node share them).
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
CPU_SAMPLE_DETS = 100000
# deterministic PT2 on the final mixed-precision space of the workload
PT_EPS2 = 1e-5
# DRAM bytes per mixed-sigma launch divided by its algorithmic bytes, from one
# ncu capture of the medium case (4.4965 GB measured / 4.4565 GB algorithmic);
# the full-size launch is too large to capture, and its traffic scales with
# the nonzeros it streams.
TRAFFIC_RATIO = 4.4965 / 4.4565


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


def make_inputs(d, case="full"):
    """case "small": the same Hamiltonian stopped after two eps1 = 1e-3
    iterations (about 8e4 determinants, a ~0.8 GB Hamiltonian: larger than L2,
    small enough for a full ncu capture)."""
    from dice_gb300 import synthetic
    if case == "small":
        return synthetic.make_workload(WORKLOAD, d, schedule=[(0, 1e-3)], maxiter=2)
    if case == "medium":  # ~5.7e5 determinants: x no longer fits L1, a few GB on the device
        return synthetic.make_workload(WORKLOAD, d, schedule=[(0, 1e-3), (2, 3e-4)], maxiter=3)
    return synthetic.make_workload(WORKLOAD, d)


def cpu_sample(work_dir, max_dets=CPU_SAMPLE_DETS):
    """Determinants for the CPU baseline: the first `max_dets` of the space the
    oracle selects with the first two eps1 = 1e-3 iterations of the workload."""
    from dice_gb300 import synthetic
    from oracle import oracle as orc
    d = os.path.join(work_dir, "cpu_sample")
    w = dict(synthetic.WORKLOADS[WORKLOAD])
    inp = synthetic.make_workload(WORKLOAD, d, schedule=[(0, 1e-3)], maxiter=2)
    run = orc.run_input(inp)
    dets = run.dets[:max_dets]
    o = orc.Oracle(os.path.join(d, "FCIDUMP"))
    t0 = time.perf_counter()
    rowptr, col, val = o.ham(dets)
    t_build = time.perf_counter() - t0
    return o, dets, len(col), t_build, w


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def time_cpu_sigma(o, n, threads, seconds=10.0, max_reps=200):
    """The oracle's restatement of the reference's rank-parallel Hmult2
    (rows dealt round-robin to `threads` workers, private accumulators,
    summed), timed on the host cores."""
    x = np.random.default_rng(1).standard_normal(n)
    o.sigma_mt(x, threads)  # warm-up
    times = []
    t_start = time.perf_counter()
    while len(times) < max_reps and (time.perf_counter() - t_start) < seconds:
        t0 = time.perf_counter()
        o.sigma_mt(x, threads)
        times.append(time.perf_counter() - t0)
    return times


def run_reference(args):
    rank, world, _ = dist_info()
    if rank != 0:
        return
    from oracle import oracle as orc
    orc.build()
    with tempfile.TemporaryDirectory() as d:
        o, dets, nnz_lower, t_build, w = cpu_sample(d)
        n = len(dets)
        threads = host_threads()
        x = np.random.default_rng(1).standard_normal(n)
        for _ in range(args.warmup):
            o.sigma_mt(x, threads)
        times = []
        for _ in range(args.steps):
            t0 = time.perf_counter()
            o.sigma_mt(x, threads)
            times.append(time.perf_counter() - t0)
    t = statistics.mean(times)
    val = n / t / 1e6
    sample = ("first %d determinants of the eps1=1e-3 space of the workload (oracle selection), "
              "lower-triangle nnz %d; the reference's rank-parallel Hmult2 (symmetric scatter in FP64, rows "
              "dealt round-robin to %d host threads standing in for its MPI ranks, private accumulators "
              "summed)" % (n, nnz_lower, threads))
    line = {"metric": "sigma Mdets/s (SHCI variational, stored H)", "value": val, "unit": "Mdets/s",
            "impl": "reference", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": t * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic",
            "config": {"workload": "mol24: synthetic molecular FCIDUMP n=24, 12a+12b, rank-72 Cholesky ERIs, seed 20260001",
                       "sample": sample},
            "cpu_baseline": {"value": val, "unit": "Mdets/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": val, "unit": "Mdets/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "Dice cannot be built here (needs Boost and MPI); the CPU oracle restating its rank-parallel "
                    "sigma is timed"}
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
        o, n, nnz_lower = cpu
        x = np.random.default_rng(3).standard_normal(n)
        x /= np.linalg.norm(x)
        t0 = time.perf_counter()
        o.rdm_on_ham(x)
        tc = time.perf_counter() - t0
        out["cpu_oracle"] = {"Gconn_s": (nnz_lower - n) / tc / 1e9, "cores": 1, "kind": "port", "seconds": tc,
                             "sample": "first %d determinants of the eps1=1e-3 space, %d connected pairs"
                                       % (n, nnz_lower - n)}
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
    """The other synthetic workloads at sizes a bench run affords, each the
    plain FP64 GPU path against the new form on the same input (final
    Davidson solve to 1e-6, loose solves at the reference's 5e-5):
    mol36 with 4 roots in block Davidson, mol64 matrix-free with 4 roots,
    mol50 with and without the learned preconditioner."""
    from dice_gb300 import engine as eng, synthetic

    def run(name, sched, maxiter, mode, block, precond="plain", basis=(0, 0), extra=()):
        inp = synthetic.make_workload(name, os.path.join(work, name), schedule=sched, maxiter=maxiter,
                                      extra=("davidsonTol 1e-6",) + tuple(extra))
        g = eng.Engine(device)
        g.set_preconditioner(precond)
        g.set_davidson_basis(*basis)
        E = g.run_input(inp, mode=mode, block=block)
        t, st, lg = g.timings(), g.run_stats(), g.run_log()
        g.close()
        return {"E_var": [float(v) for v in E], "wall_s": t["total"], "ham_s": t["ham"], "davidson_s": t["davidson"],
                "sigma_s": t["sigma"], "davidson_iters": int(st["davidson_iters"]),
                "ndets": [int(v) for v in lg["ndets"]]}

    out = {}
    sched = [(0, 1e-3)]
    ref = run("mol36", sched, 2, "fp64", True)
    new = run("mol36", sched, 2, "mixed", True, basis=(16, 12))
    out["mol36_4roots_block"] = {
        "what": "n=36, 14a+14b, 4 roots, block Davidson (k=4 per sigma launch), eps1 1e-3 x2",
        "fp64": ref, "new_form": new, "dE_per_root": [a - b for a, b in zip(new["E_var"], ref["E_var"])],
        "wall_speedup": ref["wall_s"] / new["wall_s"]}
    ref = run("mol64", [(0, 2e-3)], 1, "fp64", True, extra=("DirectDavidson",))
    new = run("mol64", [(0, 2e-3)], 1, "mixed", True, extra=("DirectDavidson",))
    out["mol64_4roots_matrix_free"] = {
        "what": "n=64, 20a+20b (two-word determinants), 4 roots, matrix-free sigma, eps1 2e-3",
        "fp64": ref, "mixed": new, "dE_per_root": [a - b for a, b in zip(new["E_var"], ref["E_var"])]}
    sched = [(0, 3e-3), (1, 7e-4)]
    plain = run("mol50", sched, 3, "mixed", False, "plain")
    mlp = run("mol50", sched, 3, "mixed", False, "mlp")
    out["mol50_learned_preconditioner"] = {
        "what": "n=50, 16a+16b, 1 root, mixed precision, reference subspace, eps1 3e-3 -> 7e-4",
        "plain": plain, "mlp": mlp, "dE": mlp["E_var"][0] - plain["E_var"][0]}
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
    e = eng.Engine(local)

    # whole variational stage, four ways: the new form (mixed precision with
    # a 16-vector Davidson subspace), the same with the learned
    # preconditioner, the plain FP64 path (the reference's algorithm), then
    # the mixed path with the reference's subspace, whose final space the
    # sigma steps below run on
    def var_run(mode, precond, basis):
        e.set_preconditioner(precond)
        e.set_davidson_basis(*basis)
        E = e.run_input(inp, mode=mode)
        return E, e.timings(), e.run_stats(), e.run_log()

    Enf, tnf, snf, lognf = var_run("mixed", "plain", (16, 8))
    Eml, tml, sml, logml = var_run("mixed", "mlp", (16, 8))
    E64, t64, s64, log64 = var_run("fp64", "plain", (0, 0))
    E32, t32, s32, log32 = var_run("mixed", "plain", (0, 0))
    N = e.ndets()
    dets_mixed = e.dets()

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
        torch.cuda.nvtx.range_push("bench_sigma_" + mode)
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
    # plain FP64 sigma on the final space of the mixed run
    nnz64, ts64, _, _, y64, alg64 = timed_sigma("fp64", x_dev, max(3, args.steps // 2), args.warmup)
    # mixed FP32 sigma (the timed region of `value`)
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

    # end to end through the C-ABI with host buffers
    for _ in range(2):
        e.sigma(x_host, "mixed")
    te = []
    for _ in range(max(3, args.steps // 2)):
        t0 = time.perf_counter()
        e.sigma(x_host, "mixed")
        te.append(time.perf_counter() - t0)
    e2e = world * k * N / statistics.mean(te) / 1e6

    peak, peak_kind = measured_peak_gbs()
    # algorithmic bytes of each launch as the library lays the matrix out
    # (k = 1 mixed: 16-bit column deltas + FP32 values, 6 B per stored entry)
    achieved = alg_bytes / t_max / 1e9
    ach64 = alg64 / statistics.mean(ts64) / 1e9

    cpu = None
    cpu_rdm = None
    if rank == 0 and not args.no_cpu:
        from oracle import oracle as orc
        orc.build()
        o, dets, nnz_lower, t_build, _ = cpu_sample(work)
        cpu_rdm = (o, len(dets), nnz_lower)
        threads = host_threads()
        tc = time_cpu_sigma(o, len(dets), threads)
        cpu = {"value": len(dets) / statistics.mean(tc) / 1e6, "unit": "Mdets/s", "cores": threads, "kind": "port",
               "sample": "first %d determinants of the eps1=1e-3 space of the workload; the oracle's restatement "
                         "of the reference's rank-parallel Hmult2 (FP64 symmetric scatter, %d host threads as "
                         "its MPI ranks), %d reps" % (len(dets), threads, len(tc))}

    line = {
        "metric": "sigma Mdets/s (SHCI variational, stored H)", "value": value, "unit": "Mdets/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64 diagonal, FP64 refinement)",
        "data": "synthetic",
        "config": {"workload": "mol24: synthetic molecular FCIDUMP n=24, 12a+12b, rank-72 Cholesky ERIs, "
                               "seed 20260001, eps1 1e-3 -> 3e-4 -> 1e-4, 1 root",
                   "n_dets": N, "nnz_offdiag": nnz, "k_vectors": k,
                   "l2": "L2 flushed between steps (256 MiB write)" if flushed else
                         "Hamiltonian (%.1f GB) larger than L2; no flush" % (nnz * 8 / 1e9),
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "e2e": {"value": e2e, "unit": "Mdets/s", "h2d_bytes_per_step": N * k * 8, "d2h_bytes_per_step": N * k * 8},
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
        "var": {"new_form": {"wall_s": tnf["total"], "E_var": float(Enf[0]), "stages_s": tnf,
                             "what": "mixed precision (FP32 sigma, float-float refinement) + 16-vector Davidson "
                                     "subspace collapsed to 8, graph-captured iterations",
                             "davidson_iters_total": snf["davidson_iters"],
                             "ndets": [int(v) for v in lognf["ndets"]],
                             "davidson_iters": [int(v) for v in lognf["davidson"]]},
                "new_form_mlp": {"wall_s": tml["total"], "E_var": float(Eml[0]), "stages_s": tml,
                                 "what": "new form + learned (BF16 MLP) preconditioner trained during the run",
                                 "davidson_iters_total": sml["davidson_iters"], "mlp_train_s": sml["t_mlp"],
                                 "davidson_iters": [int(v) for v in logml["davidson"]]},
                "mixed": {"wall_s": t32["total"], "E_var": float(E32[0]), "stages_s": t32,
                          "what": "mixed precision with the reference's Davidson subspace",
                          "davidson_iters_total": s32["davidson_iters"],
                          "ndets": [int(v) for v in log32["ndets"]], "davidson_iters": [int(v) for v in log32["davidson"]]},
                "fp64": {"wall_s": t64["total"], "E_var": float(E64[0]), "stages_s": t64,
                         "what": "plain FP64 GPU path: the reference's algorithm",
                         "davidson_iters_total": s64["davidson_iters"],
                         "ndets": [int(v) for v in log64["ndets"]], "davidson_iters": [int(v) for v in log64["davidson"]]},
                "dE_mixed_minus_fp64": float(E32[0] - E64[0]),
                "wall_speedup_mixed_vs_fp64": t64["total"] / t32["total"],
                "dE_new_form_minus_fp64": float(Enf[0] - E64[0]),
                "wall_speedup_new_form_vs_fp64": t64["total"] / tnf["total"],
                "davidson_speedup_new_form_vs_fp64": t64["davidson"] / tnf["davidson"],
                "dE_new_form_mlp_minus_fp64": float(Eml[0] - E64[0]),
                "wall_speedup_new_form_mlp_vs_fp64": t64["total"] / tml["total"]},
        "clocks": clk, "timed_wall_s": wall,
    }
    if cpu:
        line["cpu_baseline"] = cpu
    line["pt"] = pt_section(e, float(E32[0]), args.steps, rank == 0 and not args.no_cpu,
                            os.path.join(os.path.dirname(inp), "FCIDUMP"))
    line["rdm"] = rdm_section(e, nnz, cpu_rdm)
    e.close()
    if args.case == "full" and not args.no_configs:
        line["configs"] = other_configs(work, local)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


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
    ap.add_argument("--section", default="all", choices=["all", "pt"],
                    help="pt: only the variational run and the timed perturbative stage")
    ap.add_argument("--pt-eps2", type=float, default=PT_EPS2)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    elif args.section == "pt":
        run_pt_only(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

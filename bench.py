"""Benchmark: Hex8 continuity (pressure-Poisson) CVFEM assembly on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Workload (one "step"): zeroSystem + ContinuityAdvElemKernel assembly + sumInto
of a 128^3 Hex8 mesh (2,097,152 elements, 2,146,689 nodes, 57,066,625 CRS
non-zeros) with z-stretching ratio 1.05, density 1, pressure 0, dpdx 0 and a
seeded 64-mode random-Fourier velocity (|k| in [1,16], amplitude ~ k^-5/3).
The CRS values (456 MB) and node inputs exceed the 129 MB L2, so no flush
is needed between steps.  Inputs are synthetic (no dataset exists for this
path).  Printed metric: elements assembled per second (whole job).

Beside the headline number the line carries the other configurations:
"solve" (Jacobi-PCG, FP32-inner + FP64 refinement and the learned flexible CG
on the pinned 128^3 continuity system, plus "c4_192": plain vs learned at
192^3), "batch" (64 independent meshes, problems/s), "momentum_c3" (96^3
momentum assembly, its time term and the mixed-precision GMRES solve),
"heat_c1" (32^3 heat conduction assembly and solves) and
"geometry_boundary_time" (dual volume, nodal gradients with the boundary
closure, the continuity time term and the inflow/open face kernels on the
headline mesh).  --no-solve / --no-batch / --no-c1 / --no-c3 / --no-c4 /
--no-aux skip them.

--impl reference times the reference's CPU algorithm (the oracle restatement
of ContinuityAdvElemKernel + HexSCS + TpetraLinearSystem::sumInto, run on all
host cores) on the same workload and prints the same JSON line, with the
CPU Jacobi-PCG time per iteration on the full 128^3 system beside it.
Multi-GPU: replicas only (one independent mesh per rank, no collective on
the data path); value = elements of all ranks / max-over-ranks time.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Hex8 elems assembled/s; P-Poisson solve ms to 1e-8 rel-res, learned vs plain"
UNIT = "elements/s"
N_EDGE = 128


def workload_config():
    return {"workload": "continuity_adv_hex8_%d^3_zstretch1.05_fourier64" % N_EDGE, "elements": N_EDGE ** 3,
            "nodes": (N_EDGE + 1) ** 3, "nnz": (3 * N_EDGE + 1) ** 3, "kernel": "ContinuityAdvElemKernel",
            "l2": "inputs and CRS values larger than L2 (no flush)"}


def algorithmic_bytes(n_nodes, n_elems, nnz, n_rows):
    # node inputs (x 24, u 24, rho 8, p 8, Gp 24) + conn 32/elem + CRS values + rhs, counted once
    return 88 * n_nodes + 32 * n_elems + 8 * nnz + 8 * n_rows


def make_inputs():
    from nalu_gb300.meshgen import block_mesh, fourier_velocity
    c, conn, gid = block_mesh(N_EDGE, z_ratio=1.05)
    u = fourier_velocity(c, n_modes=64, kmin=1, kmax=16, seed=2024)
    n = c.shape[0]
    return c, conn, gid, u, np.ones(n), np.zeros(n), np.zeros((n, 3))


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index):
        self.index = index
        self.samples = []
        self._p = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self._p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + q,
                                        "--format=csv,noheader,nounits", "-lms", "100"],
                                       stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self._p = None
        return self

    def _read(self):
        for line in self._p.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.samples.append(parts)

    def __exit__(self, *a):
        if self._p:
            time.sleep(0.25)
            self._p.terminate()
            try:
                self._p.wait(timeout=5)
            except Exception:
                self._p.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for s in self.samples for k in range(4) if s[3 + k].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


# FP64 work of the continuity element math, FLOP per element: SASS counters
# (DADD + DMUL + 2 DFMA) of the FP64 variant of the same kernel over one
# 128^3 launch (profiles/continuity_assembly_128_fp64_flops.md)
FP64_FLOP_PER_ELEM = 2458


SM_COUNT, SMSP_PER_SM, WARP = 152, 4, 32


def compute_roof(n_elems, kernel_ms, fp64_tflops, arith="fp64", sm_mhz=None):
    """the assembly against its compute roofs.  FP64 kernel: FP64 FLOP/s over
    the measured FP64 rate.  df64 kernel: the same operations run as FP32-pair
    sequences on the FP32 pipes, so the FP64 rate is not its roof (its
    FP64-equivalent rate exceeds it by design); its roof is instruction issue,
    one warp instruction per cycle per SM sub-partition: the instructions per
    element of the committed profile of the same kernel and workload, times
    the elements, over the kernel time, against that issue rate at the
    sampled SM clock."""
    flops = FP64_FLOP_PER_ELEM * n_elems
    achieved = flops / (kernel_ms * 1e-3) / 1e12
    out = {"fp64_flop_per_element": FP64_FLOP_PER_ELEM, "fp64_equivalent_tflops": achieved,
           "fp64_peak_tflops": fp64_tflops}
    if arith == "fp64":
        out["frac_of_fp64_peak"] = achieved / fp64_tflops if fp64_tflops else None
        return out
    _, prof = profile_traffic("df64")
    ipe = prof.get("thread_instructions_per_element") if prof else None
    if ipe:
        mhz = sm_mhz or 2070.0
        peak = SM_COUNT * SMSP_PER_SM * WARP * mhz * 1e6  # thread instructions per second
        rate = ipe * n_elems / (kernel_ms * 1e-3)
        out["issue"] = {"thread_instructions_per_element": ipe, "achieved_per_s": rate, "peak_per_s": peak,
                        "frac": rate / peak, "sm_mhz": mhz,
                        "source": "instructions per element from profiles/continuity_assembly_128_df64.json"}
    return out


def solve_iteration_roof(ms, iterations, nnz, n):
    """a Jacobi-PCG iteration against HBM: the compulsory bytes of an FP64 CSR
    iteration (SpMV 12 nnz + 8 (n + 1) + 16 n, vector phase 64 n), per
    iteration time"""
    bytes_it = 12 * nnz + 8 * (n + 1) + 16 * n + 64 * n
    us = 1e3 * ms / max(1, iterations)
    gbs = bytes_it / (us * 1e-6) / 1e9
    peak, kind = peaks()
    return {"us": us, "algorithmic_bytes": bytes_it, "achieved_gbs": gbs, "frac_of_hbm": gbs / peak,
            "peak_kind": kind, "bytes_definition": "FP64 CSR (12 B per entry) + vectors, counted once"}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(arith_name):
    """DRAM bytes per assembly launch of the selected kernel from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "continuity_assembly_128%s.json" % ("_df64" if arith_name == "df64" else ""))
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("dram_bytes_per_launch"), d
    return None, None


def dist_init():
    from nalu_gb300 import replicas
    return replicas.init_from_env("gloo")


def barrier(dist):
    from nalu_gb300 import replicas
    replicas.barrier(dist)


def max_over_ranks(dist, v):
    from nalu_gb300 import replicas
    return replicas.max_over_ranks(dist, v)


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def run_cpu_sample(O, c, conn, graph, u, rho, p, gp, n_elems_sample, n_threads):
    """Oracle assembly of the first n_elems_sample elements (all nodes)."""
    rp, ci, lid = graph
    sub = np.ascontiguousarray(conn[:n_elems_sample])
    t0 = time.perf_counter()
    O.assemble(O.KERNEL_CONTINUITY_ADV, c, sub, rp, ci, lid, scalar=p, coeff=rho, vec=u, vec2=gp,
               n_threads=n_threads)
    dt = time.perf_counter() - t0
    return n_elems_sample / dt, dt


def err_over_tol(actual, expected, rowptr=None):
    """largest |a - b| / (1e-12 max(|a|,|b|) + 1e-12 scale) -- the parity
    tolerance of the tests; scale is the row's largest |entry| for CRS values
    (rowptr given), the vector's largest |entry| otherwise.  <= 1 passes."""
    if rowptr is not None:
        n = rowptr.size - 1
        rowid = np.repeat(np.arange(n), np.diff(rowptr))
        rm = np.zeros(n)
        np.maximum.at(rm, rowid, np.abs(expected))
        floor = rm[rowid]
        del rowid
    else:
        floor = np.max(np.abs(expected))
    allowed = 1e-12 * np.maximum(np.abs(actual), np.abs(expected)) + 1e-12 * floor
    return float(np.max(np.abs(actual - expected) / allowed))


class OracleChecker:
    """The oracle as the checker of the GPU results, run after every timed
    region: the FP64 CPU restatement assembles the same system, and the
    worst error ratio against the test tolerance is reported per result."""

    def __init__(self, threads):
        from oracle import oracle as O
        if not os.path.exists(os.path.join(ROOT, "oracle", "liboracle.so")):
            subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "liboracle.so"], check=True)
        self.O = O
        self.threads = threads

    def continuity(self, ctx, c, conn, gid, u, rho, p, gp):
        O = self.O
        rp, ci = ctx.graph()
        orp, oci, lid = O.graph(c.shape[0], conn, 1, gid)
        vals, rhs = ctx.system()
        t0 = time.perf_counter()
        ov, orhs = O.assemble(O.KERNEL_CONTINUITY_ADV, c, conn, rp, ci, lid, scalar=p, coeff=rho, vec=u, vec2=gp,
                              n_threads=self.threads)
        t_asm = time.perf_counter() - t0
        return {"values": err_over_tol(vals, ov, rp), "rhs": err_over_tol(rhs, orhs),
                "graph_bit_exact": bool(np.array_equal(rp, orp) and np.array_equal(ci, oci)),
                "oracle_assembly_s": t_asm, "oracle_threads": self.threads}

    def momentum(self, ctx, kernel_oracle, c, conn, gid, u, mu, rho, gju, mdot, opts):
        O = self.O
        rp, ci = ctx.graph()
        _, _, lid = O.graph(c.shape[0], conn, 3, gid)
        vals, rhs = ctx.system()
        ov, orhs = O.assemble(kernel_oracle, c, conn, rp, ci, lid, coeff=mu, vec=u, vec2=u, rho=rho, gju=gju,
                              mdot=mdot, opts=O.opts_block(**opts), n_threads=self.threads)
        return {"values": err_over_tol(vals, ov, rp), "rhs": err_over_tol(rhs, orhs)}

    def residual(self, ctx):
        """true relative residual ||b - A x|| / ||b|| of the solution, by the
        oracle's FP64 SpMV on the host copy of the system"""
        rp, ci = ctx.graph()
        vals, b = ctx.system()
        x = ctx.solution()
        r = b - self.O.spmv(rp, ci, vals, x, n_threads=self.threads)
        return float(np.linalg.norm(r) / np.linalg.norm(b))


def bench_reference(args):
    ws, rank, local, dist = dist_init()
    if rank != 0:
        return 0
    from oracle import oracle as O
    if not os.path.exists(os.path.join(ROOT, "oracle", "liboracle.so")):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "liboracle.so"], check=True)
    c, conn, gid, u, rho, p, gp = make_inputs()
    nt = cpu_threads()
    graph = O.graph(c.shape[0], conn, 1, gid)
    sample = 1 << 20  # half the mesh per step keeps the run within minutes
    for _ in range(args.warmup):
        run_cpu_sample(O, c, conn, graph, u, rho, p, gp, 1 << 16, nt)
    rates = []
    t_all = time.perf_counter()
    for _ in range(args.steps):
        r, _ = run_cpu_sample(O, c, conn, graph, u, rho, p, gp, sample, nt)
        rates.append(r)
    wall = time.perf_counter() - t_all
    value = statistics.median(rates)
    # solve half of the metric: the oracle's Jacobi-PCG (restated Belos CG + Ifpack2 Jacobi) on the full
    # 128^3 continuity system, pressure pinned at node 0, timed over a bounded number of iterations
    solve = None
    if not args.no_solve:
        rp, ci, lid = graph
        t0 = time.perf_counter()
        vals, rhs = O.assemble(O.KERNEL_CONTINUITY_ADV, c, conn, rp, ci, lid, scalar=p, coeff=rho, vec=u, vec2=gp,
                               n_threads=nt)
        t_asm = time.perf_counter() - t0
        row0 = int(lid[0])
        O.reset_rows(rp, vals, rhs, [row0])
        O.sum_into_diag(rp, ci, vals, rhs, row0, 1.0, 0.0)
        its = 200
        t0 = time.perf_counter()
        _, done, _ = O.pcg_jacobi(rp, ci, vals, rhs, tol=1e-30, max_it=its, n_threads=nt)
        t_pcg = time.perf_counter() - t0
        per_it = 1e3 * t_pcg / max(done, 1)
        solve = {"jacobi_pcg_fp64": {"ms_per_iteration": per_it, "iterations_timed": int(done), "threads": nt,
                                     "ms_for_5351_iterations": per_it * 5351},
                 "full_assembly_ms": 1e3 * t_asm,
                 "note": "5351 = iterations FP64 Jacobi-PCG needs on this system to 1e-8 (GPU run of the same "
                         "algorithm); the CPU time per iteration is measured, the total extrapolated"}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * wall / max(args.steps, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": workload_config(),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nt, "kind": "port",
                             "sample": "first %d elements of the 128^3 mesh per step, colour-parallel oracle "
                                       "(restated ContinuityAdvElemKernel + HexSCS + sumInto)" % sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "solve": solve}
    print(json.dumps(line))
    return 0


def bench_gpu(args):
    ws, rank, local, dist = dist_init()
    import nalu_gb300 as ng
    c, conn, gid, u, rho, p, gp = make_inputs()
    n_nodes, n_elems = c.shape[0], conn.shape[0]
    ctx = ng.Context(local)
    ctx.mesh_create(c, conn, gid)
    for nm, v in (("velocity", u), ("density", rho), ("pressure", p), ("dpdx", gp)):
        ctx.field_set(nm, v)
    ctx.build_elem_graph(1)
    n_rows, nnz, _ = ctx.sizes()
    # pick arithmetic x scatter by device time (both pass the parity tests)
    arith_names = {ng.ARITH_FP64: "fp64", ng.ARITH_DF64: "df64"}
    want = {"auto": (ng.ARITH_FP64, ng.ARITH_DF64), "fp64": (ng.ARITH_FP64,), "df64": (ng.ARITH_DF64,)}[args.arith]
    modes = {}
    sched = {"auto": ng.SCHEDULE_AUTO, "element": ng.SCHEDULE_ELEMENT, "ip8": ng.SCHEDULE_IP8,
             "ip16": ng.SCHEDULE_IP16}[args.schedule]
    scatters = {"auto": (ng.SCATTER_ATOMIC, ng.SCATTER_COLOURED), "atomic": (ng.SCATTER_ATOMIC,),
                "coloured": (ng.SCATTER_COLOURED,)}[args.scatter]
    for ar in want:
        for sc in scatters:
            modes["%s_%s_ms" % (arith_names[ar], {1: "atomic", 2: "coloured"}[sc])] = time_mode(ctx, ar, sc, sched=sched)
    best = min(modes, key=modes.get)
    # both arithmetics' rates, best scatter each (device time of one assembly, best of 3)
    arith_rates = {"%s_elements_per_s" % an: n_elems / (1e-3 * min(v for k, v in modes.items() if k.startswith(an)))
                   for an in arith_names.values() if any(k.startswith(an) for k in modes)}
    arith = ng.ARITH_DF64 if best.startswith("df64") else ng.ARITH_FP64
    scatter = ng.SCATTER_COLOURED if "coloured" in best else ng.SCATTER_ATOMIC
    opts = ng.default_assemble_opts(scatter=scatter, arith=arith, schedule=sched)
    # the df64 kernel's schedule (elements to threads) was autotuned by the library on its first call
    tuning = None
    if ng.ARITH_DF64 in want and sched == ng.SCHEDULE_AUTO:
        sch, sc, table = ctx.assemble_tuning(ng.KERNEL_CONTINUITY_ADV)
        tuning = {"schedule": ng.SCHEDULE_NAMES[sch], "scatter": {1: "atomic", 2: "coloured"}[sc],
                  "candidates_ms": {"%s/%s" % k: v for k, v in table.items()}}
    for _ in range(max(args.warmup, 3)):
        ctx.zero()
        ctx.assemble(ng.KERNEL_CONTINUITY_ADV, opts)
    ctx.load_complete()
    fp64_peak = ctx.probe_fp64_tflops()
    # ---- device-timed region: inputs resident in HBM ----
    launches0 = ctx.launches()
    asm_ms = []
    barrier(dist)
    ctx.synchronize()
    with ClockSampler(local) as clk:
        ctx.event_record(0)
        for s in range(args.steps):
            ctx.zero()
            ctx.event_record(2 + 2 * (s % 30))
            ctx.assemble(ng.KERNEL_CONTINUITY_ADV, opts)
            ctx.event_record(3 + 2 * (s % 30))
            if s % 30 == 29:  # event slots are reused every 30 steps
                asm_ms += [ctx.event_elapsed_ms(2 + 2 * k, 3 + 2 * k) for k in range(30)]
        ctx.event_record(1)
        ctx.synchronize()
    total_ms = ctx.event_elapsed_ms(0, 1)
    asm_ms += [ctx.event_elapsed_ms(2 + 2 * k, 3 + 2 * k) for k in range(args.steps % 30)]
    launches = ctx.launches() - launches0
    ctx.load_complete()
    barrier(dist)
    total_ms = max_over_ranks(dist, total_ms)
    value = ws * n_elems * args.steps / (total_ms * 1e-3)
    # ---- end-to-end through the C ABI with pinned host buffers ----
    pin_in = {nm: ng.PinnedArray(v.shape) for nm, v in (("coordinates", c), ("velocity", u), ("density", rho),
                                                         ("pressure", p), ("dpdx", gp))}
    for nm, v in (("coordinates", c), ("velocity", u), ("density", rho), ("pressure", p), ("dpdx", gp)):
        pin_in[nm].array[...] = v
    out_v, out_r = ng.PinnedArray((nnz,)), ng.PinnedArray((n_rows,))
    h2d = sum(a.array.nbytes for a in pin_in.values())
    d2h = out_v.array.nbytes + out_r.array.nbytes

    def e2e_step():
        # stage this step's inputs (upload stream, second field buffers), assemble
        # (waits for them in stream order), start the download of the result
        # (copy stream): the upload of step k+1 overlaps the assembly of step k,
        # the download of step k the assembly of step k+1
        for nm, a in pin_in.items():
            ctx.field_set_async_ptr(nm, a.ptr, a.array.size)
        ctx.zero()
        ctx.assemble(ng.KERNEL_CONTINUITY_ADV, opts)
        ctx.system_to_ptr_async(out_v.ptr, out_r.ptr)

    e2e_step()
    ctx.copy_wait()
    barrier(dist)
    ctx.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    ctx.copy_wait()
    ctx.synchronize()
    e2e_s = max_over_ranks(dist, time.perf_counter() - t0)
    e2e_value = ws * n_elems * args.steps / e2e_s
    # ---- plain PCG solve of the same continuity system (pressure pinned at node 0) ----
    solve = None
    # the other configurations are reported by a single-GPU run only: with N > 1
    # every rank runs the replicated headline measurement and nothing else
    extras = ws == 1
    if extras and not args.no_solve and args.solve_set == "multilevel":
        # profiling runs: the Jacobi-smoothed multigrid solve alone
        ctx.zero()
        ctx.assemble(ng.KERNEL_CONTINUITY_ADV, opts)
        ctx.reset_rows([0])
        ctx.sum_into_diag(0, 0, 1.0, 0.0)
        ctx.load_complete()
        solve = multilevel_solves(ng, ctx, learned=False)
    elif extras and not args.no_solve:
        ctx.zero()
        ctx.assemble(ng.KERNEL_CONTINUITY_ADV, opts)
        ctx.reset_rows([0])
        ctx.sum_into_diag(0, 0, 1.0, 0.0)
        ctx.load_complete()
        solve = {}
        for name, prec in (("jacobi_pcg_fp64", ng.PRECISION_FP64), ("jacobi_pcg_fp32_ir", ng.PRECISION_FP32_INNER_IR)):
            info = ctx.solve(ng.default_solver_opts(tol=1e-8, max_iters=40000, check_every=50, precision=prec),
                             raise_on_error=False)
            solve[name] = {"ms": 1e3 * info.seconds, "iterations": info.iterations,
                           "outer_iterations": info.outer_iterations, "true_rel_res": info.true_rel_res,
                           "status": info.status}
        solve["system"] = "continuity Laplacian of the same mesh, pressure pinned at node 0 (resetRows + diag 1)"
        solve["jacobi_pcg_fp64"]["per_iteration"] = solve_iteration_roof(
            solve["jacobi_pcg_fp64"]["ms"], solve["jacobi_pcg_fp64"]["iterations"], nnz, n_rows)
        # learned preconditioner: 20K pairs from PCG's first direction for 4 seeded random rhs of this
        # 128^3 system, Adam on the GPU, then flexible CG with the learned stencil
        t0 = time.perf_counter()
        ctx.learned_init(7)
        st, rf, tg = ctx.learned_harvest(n_samples=20000, n_rhs=4, seed=2024)
        t1 = time.perf_counter()
        hist = ctx.learned_train(st, rf, tg, epochs=40)
        t2 = time.perf_counter()
        learned_w = ctx.learned_weights()
        for key, probe in (("learned_fcg", 0), ("learned_fcg_probe", 1)):
            info = ctx.solve(ng.default_solver_opts(tol=1e-8, max_iters=40000, precond=ng.PRECOND_LEARNED,
                                                    learned_probe=probe), raise_on_error=False)
            solve[key] = {"ms": 1e3 * info.seconds, "setup_ms": 1e3 * info.setup_seconds,
                          "iterations": info.iterations, "learned_iterations": info.learned_iterations,
                          "fallback": info.fallback, "true_rel_res": info.true_rel_res, "status": info.status,
                          "probe_rates": [info.probe_rate_jacobi, info.probe_rate_learned]}
        solve.update(multilevel_solves(ng, ctx))
        solve["learned_fallback_codes"] = ("0 learned FCG finished, 1 it stalled -> Chebyshev-Jacobi PCG, "
                                           "2 Jacobi-CG finished (opening probe or pace bound); learned_fcg runs "
                                           "the flexible CG with the learned stencil alone, learned_fcg_probe the "
                                           "same with the opening probe; learned_multilevel uses the stencil as "
                                           "the fine-level smoother of the aggregation multigrid, "
                                           "multilevel_jacobi is that multigrid with damped-Jacobi smoothing")
        # model FLOPs of one trained sample (27 slot rows): layers 2-3 forward, dH2 and dH1, dW3 and dW2
        # (6 x 2 x 27 x 64 x 64) plus the static part of layer 1 forward and backward (2 x 2 x 64 x 81)
        flops_sample = 6 * 2 * 27 * 64 * 64 + 2 * 2 * 64 * 81
        trained = (int(0.9 * tg.size) // 256) * 256 * 40  # samples of the 40 epochs (batch 256, 10% held out)
        solve["learned_training"] = {"pairs": int(tg.size), "harvest_s": t1 - t0, "train_s": t2 - t1,
                                     "epochs": 40, "precision": "bf16 tensor cores (mma.sync m16n8k16), "
                                     "fp32 accumulation, fp32 master weights and Adam; two launches per step",
                                     "model_tflops": trained * flops_sample / (t2 - t1) * 1e-12,
                                     "val_mse_first_last": [float(hist[0, 1]), float(hist[-1, 1])]}
        solve["learned_vs_plain_time"] = solve["jacobi_pcg_fp64"]["ms"] / solve["learned_multilevel"]["ms"]
        solve["learned_stencil_fcg_vs_plain_time"] = solve["jacobi_pcg_fp64"]["ms"] / solve["learned_fcg"]["ms"]
        solve["learned_probe_vs_plain_time"] = solve["jacobi_pcg_fp64"]["ms"] / solve["learned_fcg_probe"]["ms"]
        if not args.no_c4:
            solve["c4_192"] = bench_c4(ng, learned_w, local)
    # the oracle checks every reported result after its timed region (rank 0, single GPU)
    checker = OracleChecker(cpu_threads()) if rank == 0 and ws == 1 and not args.no_cpu else None
    precision = None
    if checker is not None:
        # the headline system in both arithmetics against one FP64 oracle assembly
        for nm, v in (("velocity", u), ("density", rho), ("pressure", p), ("dpdx", gp)):
            ctx.field_set(nm, v)
        precision = {"tolerance": "|a-b| <= 1e-12 max(|a|,|b|) + 1e-12 (row max |b|); ratio <= 1 passes"}
        for an, ar in (("df64", ng.ARITH_DF64), ("fp64", ng.ARITH_FP64)):
            ctx.zero()
            ctx.assemble(ng.KERNEL_CONTINUITY_ADV, ng.default_assemble_opts(scatter=scatter, arith=ar))
            ctx.load_complete()
            precision["assembly_128_%s" % an] = checker.continuity(ctx, c, conn, gid, u, rho, p, gp)
    aux = bench_aux(ng, ctx, c, conn, rho) if extras and not args.no_aux else None
    batch = bench_batch(ng, local) if extras and not args.no_batch else None
    momentum = bench_c3(ng, local, checker=checker) if extras and not args.no_c3 else None
    heat = bench_c1(ng, local) if extras and not args.no_c1 else None
    # ---- CPU baseline on rank 0 (oracle, bounded sample) ----
    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        from oracle import oracle as O
        if not os.path.exists(os.path.join(ROOT, "oracle", "liboracle.so")):
            subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "liboracle.so"], check=True)
        sample = 1 << 18
        r, dt = run_cpu_sample(O, c, conn, O.graph(c.shape[0], conn, 1, gid), u, rho, p, gp, sample, 1)
        cpu = {"value": r, "unit": UNIT, "cores": 1, "kind": "port",
               "sample": "first %d elements of the same 128^3 workload, serial element order (%.1f s)" % (sample, dt)}
    # ---- roofline of the dominant kernel ----
    peak, peak_kind = peaks()
    alg = algorithmic_bytes(n_nodes, n_elems, nnz, n_rows)
    avg_ms = statistics.mean(asm_ms)
    achieved = alg / (avg_ms * 1e-3) / 1e9
    traffic, prof = profile_traffic(arith_names[arith])
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f64" if arith == ng.ARITH_FP64 else "f64 in/out, df64 (FP32-pair) element math",
            "fp64_elements_per_s": arith_rates.get("fp64_elements_per_s"),
            "df64_elements_per_s": arith_rates.get("df64_elements_per_s"),
            "max_err_over_tol": (None if precision is None else
                                 max(precision["assembly_128_%s" % arith_names[arith]]["values"],
                                     precision["assembly_128_%s" % arith_names[arith]]["rhs"])),
            "precision": precision,
            "data": "synthetic",
            "config": dict(workload_config(), scatter={1: "atomic", 2: "coloured"}.get(scatter, str(scatter)),
                           arith=arith_names[arith], mode_ms=modes, df64_autotune=tuning,
                           parallelism="replicas" if ws > 1 else "single"),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                         "traffic": traffic, "peak_kind": peak_kind, "algorithmic_bytes_per_launch": alg,
                         "kernel_ms": avg_ms, "fp64_probe_tflops": fp64_peak,
                         "compute": compute_roof(n_elems, avg_ms, fp64_peak, arith_names[arith],
                                                 clk.summary().get("sm_mhz"))},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "gpu_launches": launches, "clocks": clk.summary(), "cpu_baseline": cpu, "solve": solve,
            "batch": batch, "momentum_c3": momentum, "heat_c1": heat, "geometry_boundary_time": aux}
    for a in list(pin_in.values()) + [out_v, out_r]:
        a.free()
    ctx.close()
    if rank == 0:
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


HEX_SIDES = ((0, 1, 5, 4), (1, 2, 6, 5), (2, 3, 7, 6), (0, 4, 7, 3), (0, 3, 2, 1), (4, 5, 6, 7))


def timed_ms(ctx, fn, reps=5):
    fn()  # warm-up
    ms = []
    for _ in range(reps):
        ctx.event_record(0)
        fn()
        ctx.event_record(1)
        ctx.synchronize()
        ms.append(ctx.event_elapsed_ms(0, 1))
    return statistics.median(ms)


def bench_aux(ng, ctx, c, conn, rho):
    """The rows on either side of the continuity assembly, on the same 128^3
    mesh and context: dual nodal volume, the projected nodal gradient (element
    part; boundary closure over the skin), the continuity time term, and the
    inflow / open face kernels on the x = 0 / x = 1 sides."""
    n = c.shape[0]
    out = {"workload": "continuity_adv_hex8_128^3_zstretch1.05 mesh of the headline"}
    ctx.field_set("velocity_rtm", ctx.field_get("velocity", (n, 3)))
    out["mdot_ms"] = timed_ms(ctx, ctx.compute_mdot)
    o_df = ng.default_assemble_opts(arith=ng.ARITH_DF64)
    out["mdot_df64_ms"] = timed_ms(ctx, lambda: ctx.compute_mdot(o_df))
    out["dual_volume_ms"] = timed_ms(ctx, ctx.compute_dual_volume)
    out["nodal_gradient_pressure_ms"] = timed_ms(ctx, lambda: ctx.compute_nodal_gradient("pressure", "dpdx"))
    out["nodal_gradient_velocity_ms"] = timed_ms(ctx, lambda: ctx.compute_nodal_gradient("velocity", "dudx"))
    out["nodal_gradient_pressure_df64_ms"] = timed_ms(
        ctx, lambda: ctx.compute_nodal_gradient("pressure", "dpdx", arith=ng.ARITH_DF64))
    out["nodal_gradient_velocity_df64_ms"] = timed_ms(
        ctx, lambda: ctx.compute_nodal_gradient("velocity", "dudx", arith=ng.ARITH_DF64))
    t0 = time.perf_counter()
    nf = ctx.faceset_skin(0)
    out["skin_faces"] = nf
    out["skin_extraction_s"] = time.perf_counter() - t0
    out["gradient_closure_pressure_ms"] = timed_ms(ctx, lambda: ctx.nodal_gradient_boundary(0, "pressure", "dpdx"))
    ctx.field_set("density_n", 0.99 * rho)
    for lumped in (0, 1):
        o = ng.default_assemble_opts(dt=1e-3, lumped_mass=lumped)
        out["continuity_mass_%s_ms" % ("lumped" if lumped else "consistent")] = timed_ms(
            ctx, lambda: ctx.assemble(ng.KERNEL_CONTINUITY_MASS, o))
    fe, fs = ctx.faceset_get(0)
    side_nodes = np.asarray(HEX_SIDES)[fs]                       # [nf, 4] element-local
    xs = c[conn[fe[:, None], side_nodes], 0]                     # [nf, 4] x of the face nodes
    for set_id, plane in ((1, 0.0), (2, 1.0)):
        keep = np.all(np.abs(xs - plane) < 1e-12, axis=1)
        ctx.faceset_define(set_id, fe[keep], fs[keep])
        out["faces_x%d" % int(plane)] = int(keep.sum())
    ctx.field_set("cont_velocity_bc", np.tile([1.0, 0.0, 0.0], (n, 1)))
    ctx.field_set("pressure_bc", np.zeros(n))
    o = ng.default_assemble_opts()
    out["continuity_inflow_x0_ms"] = timed_ms(ctx, lambda: ctx.assemble_faces(1, ng.FACE_CONTINUITY_INFLOW, o))
    out["continuity_open_x1_ms"] = timed_ms(ctx, lambda: ctx.assemble_faces(2, ng.FACE_CONTINUITY_OPEN, o))
    return out


def bench_c1(ng, dev=0, N=32, reps=5):
    """Heat conduction (ScalarDiffElemKernel) on a 32^3 unit cube, interior
    nodes jittered +-10%, k = 1, T ~ U[0,1]; Dirichlet T = 0 at x = 0 and
    T = 1 at x = 1 (applyDirichletBCs semantics); Jacobi-PCG and
    Jacobi-GMRES(50) to 1e-8.  The whole problem fits in L2."""
    from nalu_gb300.meshgen import block_mesh
    c, conn, gid = block_mesh(N, jitter=0.1, seed=21)
    n = c.shape[0]
    T = np.random.default_rng(22).uniform(0, 1, n)
    ctx = ng.Context(dev)
    ctx.mesh_create(c, conn, gid)
    ctx.field_set("scalar_q", T)
    ctx.field_set("diff_coeff", np.ones(n))
    ctx.build_elem_graph(1)
    left, right = np.where(c[:, 0] == 0.0)[0], np.where(c[:, 0] == 1.0)[0]
    nodes = np.concatenate([left, right])
    bc = np.concatenate([np.zeros(left.size), np.ones(right.size)])
    ms = []
    for k in range(reps + 1):
        ctx.zero()
        ctx.event_record(0)
        ctx.assemble(ng.KERNEL_SCALAR_DIFF)
        ctx.event_record(1)
        ctx.synchronize()
        if k:
            ms.append(ctx.event_elapsed_ms(0, 1))
    ctx.apply_dirichlet(nodes, bc, T[nodes])
    ctx.load_complete()
    out = {"workload": "scalar_diff_hex8_32^3_jitter0.1_dirichlet_x", "elements": int(conn.shape[0]), "nodes": int(n),
           "nnz": int(ctx.sizes()[1]), "assemble_ms": statistics.median(ms),
           "elements_per_s": conn.shape[0] / (statistics.median(ms) * 1e-3)}
    for name, kw in (("jacobi_pcg_fp64", {}), ("jacobi_gmres50_fp64", {"method": ng.SOLVER_GMRES, "restart": 50})):
        info = ctx.solve(ng.default_solver_opts(tol=1e-8, max_iters=20000, **kw), raise_on_error=False)
        out[name] = {"ms": 1e3 * info.seconds, "iterations": info.iterations, "true_rel_res": info.true_rel_res,
                     "status": info.status}
    ctx.close()
    return out


def bench_c3(ng, dev=0, N=96, reps=5, checker=None):
    """Momentum (24x24 element matrices, 3 dofs/node) on a 96^3 unit cube with
    the Fourier64 velocity, viscosity 1e-3, mdot from the velocity
    (ComputeMdotElemAlgorithm): assembly time of the central
    (MomentumAdvDiffElemKernel) and the upwind-blended (MomentumUpwAdvDiff,
    alpha_upw 0.5) kernels, then the mixed-precision solve (FP32 Jacobi-GMRES(50)
    inner, FP64 refinement to 1e-8) with no-slip Dirichlet walls."""
    from nalu_gb300.meshgen import block_mesh, fourier_velocity
    c, conn, gid = block_mesh(N)
    n = c.shape[0]
    u = fourier_velocity(c, n_modes=64, kmin=1, kmax=16, seed=2024)
    ctx = ng.Context(dev)
    ctx.mesh_create(c, conn, gid)
    for nm, val in (("velocity", u), ("velocity_rtm", u), ("density", np.ones(n)), ("viscosity", np.full(n, 1e-3)),
                    ("pressure", np.zeros(n)), ("dpdx", np.zeros((n, 3))), ("dudx", np.zeros((n, 9)))):
        ctx.field_set(nm, val)
    ctx.compute_mdot()
    ctx.build_elem_graph(3)
    out = {"workload": "momentum_hex8_96^3_fourier64_mu1e-3", "elements": int(conn.shape[0]), "nodes": int(n),
           "nnz": int(ctx.sizes()[1])}
    for name, kern, kw in (("central", ng.KERNEL_MOMENTUM_ADV_DIFF, {}),
                           ("upwind_0.5", ng.KERNEL_MOMENTUM_UPW_ADV_DIFF, dict(alpha_upw=0.5, hybrid_factor=1.0))):
        out[name] = {}
        for an, ar in (("fp64", ng.ARITH_FP64), ("df64", ng.ARITH_DF64)):
            per = {}
            for sn, sc in (("atomic", ng.SCATTER_ATOMIC), ("coloured", ng.SCATTER_COLOURED)):
                o = ng.default_assemble_opts(arith=ar, scatter=sc, **kw)
                ctx.zero()
                ctx.assemble(kern, o)  # warm-up
                ms = []
                for _ in range(reps):
                    ctx.zero()
                    ctx.event_record(0)
                    ctx.assemble(kern, o)
                    ctx.event_record(1)
                    ctx.synchronize()
                    ms.append(ctx.event_elapsed_ms(0, 1))
                per[sn] = statistics.median(ms)
            best = min(per, key=per.get)  # what the scatter autotuner (NALU_SCATTER_AUTO) keeps
            out[name][an] = {"assemble_ms": per[best], "scatter": best, "scatter_ms": per,
                             "elements_per_s": conn.shape[0] / (per[best] * 1e-3)}
    # time term (MomentumMassElemKernel, BDF1)
    ctx.field_set("density_n", np.ones(n))
    ctx.field_set("velocity_n", 0.99 * u)
    out["mass"] = {}
    for lumped in (0, 1):
        o = ng.default_assemble_opts(dt=1e-3, lumped_mass=lumped)
        ms = timed_ms(ctx, lambda: ctx.assemble(ng.KERNEL_MOMENTUM_MASS, o), reps)
        out["mass"]["lumped" if lumped else "consistent"] = {"assemble_ms": ms,
                                                             "elements_per_s": conn.shape[0] / (ms * 1e-3)}
    if checker is not None:
        # df64 momentum values against the FP64 oracle (both kernels)
        mdot = ctx.field_get("mass_flow_rate_scs", (conn.shape[0], 12))
        O = checker.O
        out["precision"] = {}
        for name, kern, okern, kw in (
                ("central_df64", ng.KERNEL_MOMENTUM_ADV_DIFF, O.KERNEL_MOMENTUM_ADV_DIFF, {}),
                ("upwind_0.5_df64", ng.KERNEL_MOMENTUM_UPW_ADV_DIFF, O.KERNEL_MOMENTUM_UPW_ADV_DIFF,
                 dict(alpha_upw=0.5, hybrid_factor=1.0))):
            ctx.zero()
            ctx.assemble(kern, ng.default_assemble_opts(arith=ng.ARITH_DF64, **kw))
            out["precision"][name] = checker.momentum(ctx, okern, c, conn, gid, u, np.full(n, 1e-3), np.ones(n),
                                                      np.zeros((n, 9)), mdot, kw)
        del mdot
    ctx.zero()
    ctx.assemble(ng.KERNEL_MOMENTUM_UPW_ADV_DIFF,
                 ng.default_assemble_opts(arith=ng.ARITH_DF64, alpha_upw=0.5, hybrid_factor=1.0))
    # system of the upwind-blended kernel, no-slip walls
    on_wall = np.any((c <= 1e-12) | (c >= 1.0 - 1e-12), axis=1)
    walls = np.nonzero(on_wall)[0]
    ctx.apply_dirichlet(walls, np.zeros((walls.size, 3)), u[walls])
    ctx.load_complete()
    info = ctx.solve(ng.default_solver_opts(method=ng.SOLVER_GMRES, precision=ng.PRECISION_FP32_INNER_IR, tol=1e-8,
                                            restart=50, max_iters=20000), raise_on_error=False)
    out["solve_gmres50_fp32_ir"] = {"ms": 1e3 * info.seconds, "iterations": info.iterations,
                                    "outer_iterations": info.outer_iterations, "true_rel_res": info.true_rel_res,
                                    "status": info.status}
    if checker is not None:
        # the mixed-precision solution's residual by the oracle's FP64 SpMV
        out["solve_gmres50_fp32_ir"]["oracle_true_rel_res"] = checker.residual(ctx)
    ctx.close()
    return out


def bench_c4(ng, weights, dev=0, N=192):
    """Continuity solve on 192^3 (z-stretch 1.05, Fourier64 velocity, pressure
    pinned at node 0): plain Jacobi-PCG against flexible CG with the learned
    preconditioner trained on the 128^3 system."""
    from nalu_gb300.meshgen import block_mesh, fourier_velocity
    c, conn, gid = block_mesh(N, z_ratio=1.05)
    n = c.shape[0]
    ctx = ng.Context(dev)
    ctx.mesh_create(c, conn, gid)
    ctx.field_set("velocity", fourier_velocity(c, n_modes=64, kmin=1, kmax=16, seed=2024))
    ctx.field_set("density", np.ones(n))
    ctx.field_set("pressure", np.zeros(n))
    ctx.field_set("dpdx", np.zeros((n, 3)))
    ctx.build_elem_graph(1)
    n_rows, nnz, _ = ctx.sizes()
    E = conn.shape[0]
    # the assembly at this size (the 192^3 assembly target): both
    # arithmetics, best scatter each, device time per launch
    asm = {}
    peak, peak_kind = peaks()
    alg = algorithmic_bytes(n, E, nnz, n_rows)
    fp64_tf = ctx.probe_fp64_tflops()
    for an, ar in (("df64", ng.ARITH_DF64), ("fp64", ng.ARITH_FP64)):
        ms = min(time_mode(ctx, ar, sc) for sc in (ng.SCATTER_ATOMIC, ng.SCATTER_COLOURED))
        gbs = alg / (ms * 1e-3) / 1e9
        asm[an] = {"ms": ms, "elements_per_s": E / (ms * 1e-3), "achieved_gbs": gbs, "frac_of_hbm": gbs / peak,
                   "peak_kind": peak_kind, "compute": compute_roof(E, ms, fp64_tf, an)}
    asm["algorithmic_bytes_per_launch"] = alg
    ctx.zero()
    ctx.assemble(ng.KERNEL_CONTINUITY_ADV)
    ctx.reset_rows([0])
    ctx.sum_into_diag(0, 0, 1.0, 0.0)
    ctx.load_complete()
    ctx.learned_set_weights(weights)
    out = {"workload": "continuity_adv_hex8_192^3_zstretch1.05_fourier64, pinned node 0", "nodes": int(n),
           "nnz": int(nnz), "assembly": asm}
    info = ctx.solve(ng.default_solver_opts(tol=1e-8, max_iters=60000, check_every=50), raise_on_error=False)
    out["jacobi_pcg_fp64"] = {"ms": 1e3 * info.seconds, "iterations": info.iterations,
                              "true_rel_res": info.true_rel_res, "status": info.status}
    out.update(multilevel_solves(ng, ctx))
    out["learned_vs_plain_time"] = out["jacobi_pcg_fp64"]["ms"] / out["learned_multilevel"]["ms"]
    out["note"] = ("learned stencil alone in flexible CG at this size (not rerun): 12.4 s, 0.76x plain, "
                   "measured earlier; see the 128^3 solve block for it")
    ctx.close()
    return out


def multilevel_solves(ng, ctx, reps=2, learned=True):
    """The continuity system of ctx through the aggregation multigrid in
    flexible CG: learned fine-level smoother (the learned preconditioner) and
    damped-Jacobi smoothing (the same method without the network); best of
    reps calls, each building its hierarchy (set-up included in ms)."""
    out = {}
    variants = (("learned_multilevel", ng.PRECOND_LEARNED_MULTILEVEL),) if learned else ()
    for key, pc in variants + (("multilevel_jacobi", ng.PRECOND_MULTILEVEL),):
        best = None
        for _ in range(reps):
            info = ctx.solve(ng.default_solver_opts(tol=1e-8, max_iters=5000, check_every=10, precond=pc),
                             raise_on_error=False)
            if best is None or info.seconds < best.seconds:
                best = info
        rows, nnz = ctx.multilevel_levels()
        out[key] = {"ms": 1e3 * best.seconds, "setup_ms": 1e3 * best.setup_seconds, "iterations": best.iterations,
                    "true_rel_res": best.true_rel_res, "status": best.status, "level_rows": rows,
                    "operator_complexity": sum(nnz) / nnz[0] if nnz else None}
    if learned:
        out["learned_smoother_iteration_gain"] = out["multilevel_jacobi"]["iterations"] / max(
            1, out["learned_multilevel"]["iterations"])
    return out


def bench_batch(ng, dev=0, n_problems=64, seed=2025, reps=2):
    """64 independent continuity problems (edges per axis log-uniform in
    [16, 96], interior jitter 10%, own Fourier velocity each, pressure pinned
    at each problem's first node): one assembly launch over the union mesh,
    then one persistent Jacobi-CG launch with per-problem scalars, to 1e-8."""
    from nalu_gb300.meshgen import batch_block_meshes, fourier_velocity
    c, conn, gid, off, edges = batch_block_meshes(n_problems, edge_range=(16, 96), jitter=0.1, seed=seed)
    n = c.shape[0]
    u = np.concatenate([fourier_velocity(c[off[k]:off[k + 1]], n_modes=64, seed=seed + 1 + k)
                        for k in range(n_problems)])
    ctx = ng.Context(dev)
    ctx.mesh_create(c, conn, gid)
    ctx.field_set("velocity", u)
    ctx.field_set("density", np.ones(n))
    ctx.field_set("pressure", np.zeros(n))
    ctx.field_set("dpdx", np.zeros((n, 3)))
    ctx.build_elem_graph(1)
    ctx.set_problems(off)
    pins = off[:-1]
    # assemble once and time the tile sizes of the batched solve (autotuner)
    ctx.zero()
    ctx.assemble(ng.KERNEL_CONTINUITY_ADV)
    ctx.reset_rows(pins)
    for q in pins:
        ctx.sum_into_diag(int(q), 0, 1.0, 0.0)
    ctx.load_complete()
    tile_rows, tile_ms = ctx.batch_autotune(100)
    best = None
    for _ in range(reps):
        ctx.synchronize()
        t0 = time.perf_counter()
        ctx.event_record(0)
        ctx.zero()
        ctx.assemble(ng.KERNEL_CONTINUITY_ADV)
        ctx.reset_rows(pins)
        for q in pins:
            ctx.sum_into_diag(int(q), 0, 1.0, 0.0)
        ctx.load_complete()
        ctx.event_record(1)
        infos = ctx.solve_batched(ng.default_solver_opts(tol=1e-8, max_iters=40000), raise_on_error=False)
        ctx.synchronize()
        wall = time.perf_counter() - t0
        asm_ms = ctx.event_elapsed_ms(0, 1)
        if best is None or wall < best[0]:
            best = (wall, asm_ms, infos)
    wall, asm_ms, infos = best
    its = sorted(i.iterations for i in infos)
    nnz = ctx.sizes()[1]
    out = {"workload": "64 continuity problems, edges log-U[16,96] per axis, jitter 0.1, Fourier64 each",
           "problems": n_problems, "elements": int(conn.shape[0]), "nodes": int(n), "nnz": int(nnz),
           "problems_per_s": n_problems / wall, "per_problem_ms": 1e3 * wall / n_problems,
           "wall_ms": 1e3 * wall, "assemble_bc_ms": asm_ms, "solve_ms": infos[0].seconds * 1e3,
           "iterations_min_median_max": [its[0], its[len(its) // 2], its[-1]],
           "max_true_rel_res": max(i.true_rel_res for i in infos),
           "all_converged": all(i.status == 0 for i in infos), "preconditioner": "jacobi (plain PCG)",
           "tile_autotune": {"rows_per_tile": tile_rows, "ms_per_iteration": {str(k): v for k, v in tile_ms.items()}}}
    # learned flexible CG on the same batch: weights trained on this union system
    # (20K PCG first-direction pairs, 4 seeded rhs, 40 epochs); the solve time
    # includes the stencil set-up of the problems that try it, the training is
    # reported beside it
    t0 = time.perf_counter()
    ctx.learned_init(7)
    st, rf, tg = ctx.learned_harvest(n_samples=20000, n_rhs=4, seed=2026)
    t1 = time.perf_counter()
    ctx.learned_train(st, rf, tg, epochs=40)
    train_s = time.perf_counter() - t0
    train_only_s = time.perf_counter() - t1
    linfos = None
    for _ in range(reps):  # the same repetitions as the plain solve, fastest kept
        li = ctx.solve_batched(ng.default_solver_opts(tol=1e-8, max_iters=40000, precond=ng.PRECOND_LEARNED),
                               raise_on_error=False)
        if linfos is None or li[0].seconds < linfos[0].seconds:
            linfos = li
    lits = sorted(i.iterations for i in linfos)
    lsolve = linfos[0].seconds
    out["learned_fcg"] = {"solve_ms": 1e3 * lsolve, "setup_ms": 1e3 * linfos[0].setup_seconds,
                          "problems_per_s": n_problems / (asm_ms * 1e-3 + lsolve),
                          "iterations_min_median_max": [lits[0], lits[len(lits) // 2], lits[-1]],
                          "problems_on_learned": int(sum(i.fallback == 0 for i in linfos)),
                          "problems_with_learned_iterations": int(sum(i.learned_iterations > 0 for i in linfos)),
                          "problems_probe_chose_jacobi": int(sum(i.fallback == 2 for i in linfos)),
                          "problems_fell_back_after_stall": int(sum(i.fallback == 1 for i in linfos)),
                          "max_true_rel_res": max(i.true_rel_res for i in linfos),
                          "all_converged": all(i.status == 0 for i in linfos), "training_s": train_s,
                          "train_only_s": train_only_s}
    out["learned_vs_plain_time"] = infos[0].seconds / lsolve
    # the multigrid preconditioner per problem: one hierarchy for the union
    # (block diagonal), flexible CG with per-problem scalars and stop tests
    minfos = None
    for _ in range(reps):
        mi = ctx.solve_batched(ng.default_solver_opts(tol=1e-8, max_iters=40000, precond=ng.PRECOND_MULTILEVEL),
                               raise_on_error=False)
        if minfos is None or mi[0].seconds < minfos[0].seconds:
            minfos = mi
    mits = sorted(i.iterations for i in minfos)
    out["multilevel_fcg"] = {"solve_ms": 1e3 * minfos[0].seconds, "setup_ms": 1e3 * minfos[0].setup_seconds,
                             "problems_per_s": n_problems / (asm_ms * 1e-3 + minfos[0].seconds),
                             "iterations_min_median_max": [mits[0], mits[len(mits) // 2], mits[-1]],
                             "max_true_rel_res": max(i.true_rel_res for i in minfos),
                             "all_converged": all(i.status == 0 for i in minfos)}
    out["multilevel_vs_plain_time"] = infos[0].seconds / minfos[0].seconds
    out.update(batch_multilevel(ng, ctx, off, asm_ms))
    ctx.close()
    return out


def batch_multilevel(ng, ctx, off, asm_ms):
    """The whole batch as one block-diagonal system through the multilevel
    flexible CG (aggregation never crosses problems: they share no
    couplings).  The union tolerance is tightened to 0.9e-8 min_k ||b_k|| / ||b||
    so that every problem meets 1e-8; each problem's true residual is checked
    after the solve (FP64 SpMV on the device, norms per problem on the host)."""
    import ctypes
    n_rows = ctx.sizes()[0]
    b = np.zeros(n_rows)
    if ng.lib().nalu_linsys_copy(ctx.handle, None, b.ctypes.data_as(ctypes.c_void_p), 0) != 0:
        raise RuntimeError("rhs copy failed")
    seg = np.add.reduceat(b * b, off[:-1])
    bk = np.sqrt(seg)
    tol_u = 0.9e-8 * float(np.min(bk[bk > 0])) / float(np.linalg.norm(b))
    out = {}
    for key, pc in (("multilevel_jacobi_union", ng.PRECOND_MULTILEVEL),
                    ("learned_multilevel_union", ng.PRECOND_LEARNED_MULTILEVEL)):
        best = None
        for _ in range(2):
            info = ctx.solve(ng.default_solver_opts(tol=tol_u, max_iters=5000, check_every=10, precond=pc),
                             raise_on_error=False)
            if best is None or info.seconds < best.seconds:
                best = info
        x = ctx.solution()
        r = b - ctx.spmv(x)
        rk = np.sqrt(np.add.reduceat(r * r, off[:-1])) / np.where(bk > 0, bk, 1.0)
        out[key] = {"solve_ms": 1e3 * best.seconds, "setup_ms": 1e3 * best.setup_seconds,
                    "iterations": best.iterations, "union_tol": tol_u, "status": best.status,
                    "max_problem_true_rel_res": float(np.max(rk)), "all_problems_converged": bool(np.all(rk <= 1e-8)),
                    "problems_per_s": len(bk) / (asm_ms * 1e-3 + best.seconds)}
    return out


def time_mode(ctx, arith, scatter, reps=3, sched=0):
    """Device time (ms, best of reps after one warm-up) of one continuity assembly."""
    import nalu_gb300 as ng
    o = ng.default_assemble_opts(scatter=scatter, arith=arith, schedule=sched)
    best = None
    for r in range(reps + 1):
        ctx.zero()
        ctx.event_record(62)
        ctx.assemble(ng.KERNEL_CONTINUITY_ADV, o)
        ctx.event_record(63)
        ms = ctx.event_elapsed_ms(62, 63)
        if r > 0 and (best is None or ms < best):
            best = ms
    ctx.load_complete()
    return best


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-solve", action="store_true")
    ap.add_argument("--solve-set", default="all", choices=["all", "multilevel"],
                    help="solves on the headline system: all, or the Jacobi-smoothed multigrid alone (profiling)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the 64-problem batched workload")
    ap.add_argument("--no-c4", action="store_true", help="skip the 192^3 learned-vs-plain continuity solve")
    ap.add_argument("--no-c3", action="store_true", help="skip the 96^3 momentum assembly and solve")
    ap.add_argument("--no-c1", action="store_true", help="skip the 32^3 heat-conduction assembly and solve")
    ap.add_argument("--no-aux", action="store_true",
                    help="skip the geometry / gradient / time-term / face-kernel timings on the headline mesh")
    ap.add_argument("--size", type=int, default=128, help="elements per edge (default: the 128^3 workload)")
    ap.add_argument("--arith", default="auto", choices=["auto", "fp64", "df64"],
                    help="element-math arithmetic (auto: the faster; both pass the parity tests)")
    ap.add_argument("--schedule", default="auto", choices=["auto", "element", "ip8", "ip16"],
                    help="df64 kernel schedule (auto: the library's autotuner)")
    ap.add_argument("--scatter", default="auto", choices=["auto", "atomic", "coloured"],
                    help="scatter of the headline assembly (auto: the faster)")
    args = ap.parse_args()
    global N_EDGE
    N_EDGE = args.size
    if args.impl == "reference":
        return bench_reference(args)
    return bench_gpu(args)


if __name__ == "__main__":
    sys.exit(main())

#!/usr/bin/env python
"""Benchmark: excitonic-Hamiltonian build (+ gradient) seconds per optimizer iteration.

One step = one optimizer iteration of the state optimisation on a seeded synthetic dimer:
transition densities of both fragments from the current states, the order-0 XR-H build,
its lowest eigenpair (FP64), and the energy gradient (state coefficients and orbital
rotations) when the adjoint is enabled.  `value` is device-resident (inputs in HBM);
`e2e` goes through the same public API with the states in pinned host memory and the
energy/gradient copied back every step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--config 3|1] [--precision P]
  python bench.py --impl reference ...   (the FP64 CPU oracle on the host cores)
  python bench.py --config 2 ...         (trimer: pair builds + matrix-free H x v Lanczos ground state)

The default workload is the dimer 2 x 14 spatial orbitals / 60 states per charge sector
(build + state and orbital gradient + step); --config 1 is the 2 x 9 / 10-state dimer.

Multi-GPU: the path does not shard (one dimer), so N>1 runs N independent replicas
(one per rank, launched by torchrun); value = max time over ranks / iterations of all ranks
(replica_aggregate).
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

CONFIGS = {
    2: dict(n_orb=14, n_states=40, n_frag=3,
            name="linear trimer 3x14 spatial orbitals (28 spin orbitals each), 40 states per charge sector "
                 "(+1,0,-1), neutral sector of the product space (448 000 states), matrix-free H x v"),
    1: dict(n_orb=9, n_states=10, name="dimer 2x9 spatial orbitals (18 spin orbitals each), 10 states per charge "
                                      "sector (+1,0,-1; 3/4/5 electrons), order-0 XR-H 900x900"),
    3: dict(n_orb=14, n_states=60, name="dimer 2x14 spatial orbitals (28 spin orbitals each), 60 states per charge "
                                       "sector (+1,0,-1), order-0 XR-H 32400x32400"),
    4: dict(n_orb=14, n_states=100, n_frag=8,
            name="ring of 8 fragments x 14 spatial orbitals (28 spin orbitals each), 100 states per charge sector "
                 "(+1,0,-1): all 28 pairs (neutral sectors, 30 000 states, with the state gradient of the pair "
                 "expansion) and the 8 nearest-neighbour triples (neutral sectors, 7 000 000 states, matrix-free "
                 "H x v)"),
}
SEED = 1234
METRIC = "XR-H build+grad s/iter vs plain FP64 GPU, at |dE|<=1e-6 Eh vs FP64 oracle"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--config", type=int, default=3, choices=sorted(CONFIGS))
    p.add_argument("--precision", default="tf32x3")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-variants", action="store_true")
    p.add_argument("--states", type=int, default=None, help="states per charge sector (default: the config's)")
    p.add_argument("--orbitals", type=int, default=None, help="spatial orbitals per fragment (default: the config's)")
    p.add_argument("--no-triples", action="store_true", help="ring (config 4): pairs and monomers only")
    return p.parse_args()


def make_system(cfg, states=None, orbitals=None):
    """The seeded dimer of a config; states / orbitals override the states per charge sector
    and the spatial orbitals per fragment (smaller cases of the same kernels, e.g. for
    profiler captures)."""
    from qodeapplications_gb300 import synthetic as S
    c = CONFIGS[cfg]
    return S.make_system(n_frag=2, n_orb=orbitals or c["n_orb"], n_states=states or c["n_states"],
                         charges=(+1, 0, -1), seed=SEED)


def workload_name(args):
    name = CONFIGS[args.config]["name"]
    if args.config != 2 and (args.states or args.orbitals):
        c = CONFIGS[args.config]
        if args.states:
            name = name.replace(f"{c['n_states']} states", f"{args.states} states")
        if args.orbitals:
            name = name.replace(f"2x{c['n_orb']} spatial orbitals ({2 * c['n_orb']} spin",
                                f"2x{args.orbitals} spatial orbitals ({2 * args.orbitals} spin")
        name = name.split(", order-0")[0]
    return name


# ------------------------------------------------------------------------------------------
# CPU oracle step (reference arm and cpu_baseline)
# ------------------------------------------------------------------------------------------

def _oracle():
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import xr_oracle as O
    return O


def oracle_step(sysd):
    """One full FP64 build with the NumPy oracle (the reference's algorithm and contraction
    order): densities of both fragments (ccaa included, as build_density_tensors.py:122-133
    builds them), the order-0 XR-H (get_xr_result.py:86-132), the dense eigensolve
    (mains/workflow.py:229).  Returns (E0, seconds of densities, seconds of H, seconds of
    the eigensolve)."""
    import numpy as np
    O = _oracle()
    charges = list(sysd["charges"])
    ints = O.FragInts(sysd["h"], sysd["V"], sysd["Ns"])
    t0 = time.perf_counter()
    dens = [O.build_densities({c: O.Sector(*sysd["states"][m][c]) for c in charges}, sysd["n_orb"],
                              sysd["n_core"], sysd["n_elec_ref"]) for m in range(2)]
    t1 = time.perf_counter()
    H1, H2 = O.get_xr_H0(ints, dens, [charges, charges])
    H = O.full_H(H1, H2)
    t2 = time.perf_counter()
    w = np.linalg.eigvalsh(H)
    t3 = time.perf_counter()
    return float(w[0]), t1 - t0, t2 - t1, t3 - t2


def _einsum_rate(n_rows, K, N, reps=2):
    """FP64 GFLOP/s of the host BLAS on one precontraction-shaped product (n_rows x K) @ (K x N),
    the dominant contraction shape of the reference's H build (precontract.py:75)."""
    import numpy as np
    rng = np.random.default_rng(0)
    A = rng.standard_normal((n_rows, K))
    B = rng.standard_normal((K, N))
    best = None
    for _ in range(reps):
        t0 = time.perf_counter()
        A @ B
        dt = time.perf_counter() - t0
        best = dt if best is None else min(best, dt)
    return 2.0 * n_rows * K * N / best / 1e9


def oracle_sampled_iteration(sysd, h_flops, budget_s=20.0):
    """Extrapolated FP64 CPU seconds of one build of the reference's algorithm at a size where
    a full CPU run takes hours (the 2 x 14 / 60-state dimer), from a bounded sample:

    * densities (the dominant CPU cost): every (op, bra charge, ket charge) block the reference
      builds (build_density_tensors.py:57-160, ccaa included) is built by the oracle for a
      random subset of the ket configurations (the work is a sum over ket configurations, so
      it scales with their number) and two bra-state counts (it is linear in them); the time
      is extrapolated to all configurations and all states, for both fragments;
    * H: the algorithmic FLOPs of the order-0 build (precontractions, final contractions, and
      the n^2 N^4 monomer_2e contraction of every stored ccaa block) divided by the host BLAS
      rate on a precontraction-shaped product;
    * the dense eigensolve of the full product-basis H (mains/workflow.py:229): symmetric
      eigvalsh timed at a smaller dimension and scaled by n^3 (a lower bound of the reference's
      general scipy.linalg.eig).
    The gradient is not included (the reference's costs two more H builds with determinant
    densities, state_gradients.py:170-185): the figure is a lower bound of a CPU iteration."""
    import numpy as np
    O = _oracle()
    rng = np.random.default_rng(5)
    charges = list(sysd["charges"])
    n_orb, n_core = sysd["n_orb"], sysd["n_core"]
    N = 2 * n_orb
    st = sysd["states"][0]
    blocks = [(op, bc, kc) for bc in charges for kc in charges for op in O.OPS_FOR_DCHG.get(bc - kc, ())]
    per_block_budget = budget_s / len(blocks)
    dens_s, detail = 0.0, {}
    for (op, bc, kc) in blocks:
        zb, mb = st[bc]
        zk, mk = st[kc]
        n_b = zb.shape[0]
        frac = min(1.0, {1: 0.2, 2: 0.1, 3: 0.03, 4: 0.004}[len(op)])
        n_sub = max(8, int(frac * len(mk)))
        sub = np.sort(rng.choice(len(mk), size=min(n_sub, len(mk)), replace=False))
        nbs = (1, 2) if len(op) == 4 else (2, 4)
        ts = []
        for nb in nbs:
            t0 = time.perf_counter()
            O.transition_density(op, zb[:nb], mb, zk[:, sub], mk[sub], N, n_orb, n_core)
            ts.append(time.perf_counter() - t0)
        slope = max(0.0, (ts[1] - ts[0]) / (nbs[1] - nbs[0]))
        t_full = (ts[0] + slope * (n_b - nbs[0])) * len(mk) / len(sub)
        detail[f"{op}({bc},{kc})"] = round(t_full, 3)
        dens_s += t_full
        if sum(ts) > per_block_budget:
            per_block_budget = max(0.5, per_block_budget * 0.8)
    dens_s *= 2                            # both fragments have the same sizes
    # monomer_2e on every stored ccaa block: n_b n_k N^4 multiply-adds per charge, both fragments
    n = {c: st[c][0].shape[0] for c in charges}
    mono_flops = 2 * sum(2.0 * n[c] * n[c] * N ** 4 for c in charges)
    rate = _einsum_rate(n[charges[0]] ** 2, N * N, N * N)
    h_s = (h_flops + mono_flops) / (rate * 1e9)
    # dense eigensolve of the whole product-basis H
    dim = sum(n.values()) ** 2
    m_s = 2000
    A = rng.standard_normal((m_s, m_s))
    A = A + A.T
    t0 = time.perf_counter()
    np.linalg.eigvalsh(A)
    eig_s = (time.perf_counter() - t0) * (dim / m_s) ** 3
    return dict(total=dens_s + h_s + eig_s, densities=dens_s, h_build=h_s, eigensolve=eig_s,
                blas_gflops=rate, density_blocks_fragment0_s=detail)


def time_oracle(sysd, budget_s=30.0):
    t0 = time.perf_counter()
    e, td, th, te = oracle_step(sysd)
    dt = time.perf_counter() - t0
    return dt, e, dict(densities=td, h_build=th, eigensolve=te)


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count()


# ------------------------------------------------------------------------------------------
# GPU path
# ------------------------------------------------------------------------------------------

class ClockSampler:
    def __init__(self, path):
        self.path, self.proc = path, None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self, device_index):
        import statistics
        sm, mx, reasons = [], [], set()
        try:
            for line in open(self.path):
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9 or parts[0] != str(device_index):
                    continue
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
                for name, val in zip(["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"],
                                     parts[5:9]):
                    if val.lower().startswith("active"):
                        reasons.add(name)
        except (OSError, ValueError):
            pass
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


class GPUIteration:
    """Device-resident optimizer iteration (qodeapplications_gb300.iteration.XRStateOptimizer):
    densities -> H -> lowest eigenpair (FP64 Lanczos) -> state and orbital gradients -> state step."""

    def __init__(self, sysd, precision):
        import torch
        from qodeapplications_gb300.iteration import XRStateOptimizer
        self.torch = torch
        self.opt = XRStateOptimizer(sysd, precision=precision)
        self.charges = list(sysd["charges"])
        self.host = [{c: torch.as_tensor(sysd["states"][m][c][0]).pin_memory() for c in self.charges}
                     for m in range(2)]
        self.h2d_bytes = sum(t.numel() * 8 for d in self.host for t in d.values())
        self.E_host = torch.empty(1, dtype=torch.float64).pin_memory()
        n_g = sum(t.numel() for d in self.host for t in d.values())
        self.g_host = torch.empty(n_g, dtype=torch.float64).pin_memory()
        self.d2h_bytes = 8 + n_g * 8

    def step(self):
        return self.opt.iterate()

    def step_e2e(self):
        """Through host buffers: states from pinned host memory in, energy and the updated
        states (the optimizer's output) back to pinned host memory."""
        torch = self.torch
        for m in (0, 1):
            for c in self.charges:
                self.opt.plan.coeffs[m][c].copy_(self.host[m][c], non_blocking=True)
        e = self.opt.iterate()
        off = 0
        for m in (0, 1):
            for c in self.charges:
                z = self.opt.plan.coeffs[m][c].reshape(-1)
                self.g_host[off:off + z.numel()].copy_(z, non_blocking=True)
                off += z.numel()
        torch.cuda.current_stream().synchronize()
        return e


def graph_launches(it):
    """Kernels of this library launched per replayed iteration (counted while capturing)."""
    return getattr(it.opt, "graph_kernels", None)


def time_variant(sysd, precision, steps, warmup, l2_flush):
    """Device-resident seconds per iteration of one precision variant; returns (s/iter, E list, it)."""
    import torch
    it = GPUIteration(sysd, precision)
    for _ in range(max(warmup, 3)):
        it.step()
    torch.cuda.synchronize()
    ms, Es = [], []
    for _ in range(steps):
        l2_flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        Es.append(it.step())
        e1.record()
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    return sum(ms) / 1e3 / steps, Es, it


# DRAM bytes (read + write) per launch of the dominant kernel, from ncu captures of the bench
# command (the summaries are in profiles/); None where no capture of the current kernel exists
DENSITY_ADJ_TRAFFIC = {(3, "density_adjoint_f32_grouped_kernel"): 0.675e9}


def measure_peaks():
    """Throughput of the arithmetic pipes the SIMT kernels use, measured live like the HBM and
    BF16 figures of MEASURED_PEAKS.json: the best of 3 CUDA-event-timed torch.matmul calls
    (cuBLAS) per type -- FP64 (4096^3), FP32 with IEEE products (8192^3, the CUDA-core FMA
    rate) and TF32 tensor-core (8192^3).  No clock or power setting is touched."""
    import torch
    out = {}
    prev = torch.get_float32_matmul_precision()
    for name, dtype, n, prec in (("fp64_tflops", torch.float64, 4096, None),
                                 ("fp32_simt_tflops", torch.float32, 8192, "highest"),
                                 ("tf32_tflops", torch.float32, 8192, "high")):
        if prec:
            torch.set_float32_matmul_precision(prec)
        a = torch.randn(n, n, dtype=dtype, device="cuda")
        b = torch.randn(n, n, dtype=dtype, device="cuda")
        a @ b
        torch.cuda.synchronize()
        best = None
        for _ in range(3):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            a @ b
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        out[name] = 2.0 * n ** 3 / (best * 1e-3) / 1e12
        del a, b
    torch.set_float32_matmul_precision(prev)
    torch.cuda.empty_cache()
    out["how"] = "torch.matmul (cuBLAS), best of 3, CUDA events: fp64 4096^3, fp32 IEEE 8192^3, tf32 8192^3"
    return out


def density_adjoint_work(adj, m):
    """Algorithmic bytes and FLOPs of one FP32 density-adjoint launch of fragment m (all its
    accumulated blocks): coupling lists read once (P, Q 4 B and sign 1 B per coupling, idx_ptr
    8 B per index), dE/drho read once (8 B per element), the FP32 coefficient rows read once and
    the FP32 gradient rows read and written once; 4 n_b n_k FLOPs per coupling (U = zb^T G and
    W = G zk)."""
    plan = adj.plan
    sp = plan.spaces[m]
    bld = plan.builders[m]
    by, fl = 0.0, 0.0
    for (mm, op, bc, kc, cp, rt, grho, gT) in adj.dens_adj_all:
        if mm != m:
            continue
        nb, nk = rt.shape[0], rt.shape[1]
        by += 8.0 * (cp.K + 1) + 9.0 * cp.count + 8.0 * cp.K * nb * nk
        fl += 4.0 * nb * nk * cp.count
    for c in sp.charges:
        by += 4.0 * sp.n_conf[c] * bld.zT32[c].shape[1] + 8.0 * sp.n_conf[c] * plan.n_states[m][c]
    return by, fl


def dominant_kernel_roofline(it, config, reps=20):
    """Live CUDA-event timing, on the launching stream, of the dominant kernel of the step in
    the ncu launch list: the FP32 density adjoint (dE/dz from dE/drho), one launch per
    fragment (lane per coupling on unit tables for blocks of at most 16 states, one CTA per
    operator index above).  Timed with the buffers the last iteration left (the launches add
    into the gradient buffers, which the next iteration zeroes)."""
    import torch
    from qodeapplications_gb300 import _lib
    adj = it.opt.adj
    launches = []
    for m, (tasks, n_t, units, n_u, mx) in enumerate(getattr(adj, "dens_adj_units", ())):
        launches.append(("xrh_density_adjoint_f32_units", (_lib.ptr(tasks), n_t, _lib.ptr(units), n_u, mx, 1)))
    for (tasks, n_t, ctas, mnb, mnk) in adj.dens_adj_groups:
        launches.append(("xrh_density_adjoint_f32_grouped", (_lib.ptr(tasks), n_t, ctas, mnb, mnk)))
    if not launches:
        return None
    name = launches[0][0]
    launches = [l for l in launches if l[0] == name]
    work = [density_adjoint_work(adj, m) for m in (0, 1)]
    stream = torch.cuda.current_stream()
    s = _lib.stream_ptr(stream)
    for _ in range(3):
        for fn, a in launches:
            _lib.call(fn, *a, s)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        for fn, a in launches:
            _lib.call(fn, *a, s)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / (reps * len(launches))
    by = sum(w[0] for w in work) / len(work)
    fl = sum(w[1] for w in work) / len(work)
    kname = ("density_adjoint_units_kernel" if name.endswith("units") else "density_adjoint_f32_grouped_kernel")
    return dict(name=f"{kname} (FP32 density adjoint, one launch per fragment)", ms=ms, bytes=by, flops=fl,
                kernel=kname, traffic=DENSITY_ADJ_TRAFFIC.get((config, kname)))


def replica_aggregate(total_ms, e2e_ms, steps, world, device):
    """Whole-job figures of N independent replicas: every rank ran `steps` iterations of its
    own copy of the workload; the job's time is the slowest rank's (max over ranks), so the
    job's seconds per iteration are that time over the iterations of all ranks.  Returns
    (max total ms, max e2e ms, job s/iter, job e2e s/iter)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([total_ms, e2e_ms], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    mx, me = float(t[0]), float(t[1])
    return mx, me, mx / 1e3 / (steps * world), me / 1e3 / (steps * world)


def run_ours(args):
    import torch
    import torch.distributed as dist
    from qodeapplications_gb300 import _lib
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    sysd = make_system(args.config, args.states, args.orbitals)
    l2_flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    it = GPUIteration(sysd, args.precision)
    for _ in range(max(args.warmup, 3)):
        it.step()
    barrier()
    clock_path = os.path.join(tempfile.gettempdir(), f"xrh_clocks_{os.getpid()}.csv")
    step_ms, energies = [], []
    _lib.LaunchCounter.count = 0
    with ClockSampler(clock_path) as cs:
        # NVTX range "xrh_timed" marks the timed iterations for profilers (ncu --nvtx-include)
        torch.cuda.nvtx.range_push("xrh_timed")
        for _ in range(args.steps):
            l2_flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            energies.append(it.step())
            e1.record()
            torch.cuda.synchronize()
            step_ms.append(e0.elapsed_time(e1))
        torch.cuda.nvtx.range_pop()
        barrier()
    eager_calls = _lib.LaunchCounter.count
    per_iter = graph_launches(it) or 0
    launches = eager_calls + per_iter * args.steps
    clocks = cs.summary(local)
    total_ms = sum(step_ms)

    # end to end through host buffers (fresh optimizer state each step: same work per step)
    barrier()
    e2e_ms = []
    for _ in range(args.steps):
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        it.step_e2e()
        t1.record()
        torch.cuda.synchronize()
        e2e_ms.append(t0.elapsed_time(t1))
    e2e_total = sum(e2e_ms)

    total_ms, e2e_total, s_per_iter, e2e_s_per_iter = replica_aggregate(total_ms, e2e_total, args.steps, world,
                                                                        "cuda")
    h2d_bytes, d2h_bytes = it.h2d_bytes, it.d2h_bytes
    residual_last, flops_per_build = it.opt.residual, it.opt.plan.flops
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return

    peaks = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(HERE, "MEASURED_PEAKS.json")) else {}
    live = measure_peaks()
    dk = dominant_kernel_roofline(it, args.config)
    if dk is not None:
        hbm = float(peaks.get("hbm_gbs", 6800.0))
        gbs = dk["bytes"] / (dk["ms"] * 1e-3) / 1e9
        tflops = dk["flops"] / (dk["ms"] * 1e-3) / 1e12
        roofline = {"bound": "fp32 (CUDA-core FMA)", "kernel": dk["name"], "achieved": tflops,
                    "peak": live["fp32_simt_tflops"], "unit": "TFLOP/s", "frac": tflops / live["fp32_simt_tflops"],
                    "traffic": dk["traffic"], "launch_ms": dk["ms"],
                    "algorithmic_bytes_per_launch": dk["bytes"], "flops_per_launch": dk["flops"],
                    "peak_source": "fp32 IEEE cuBLAS GEMM measured in this run (of measured)",
                    "hbm": {"achieved_gbs": gbs, "peak_gbs": hbm, "frac": gbs / hbm,
                            "peak_source": "MEASURED_PEAKS.json hbm_gbs (of measured)" if "hbm_gbs" in peaks
                            else "fallback 6.8 TB/s (of fallback)"},
                    "traffic_source": ("ncu dram__bytes_read.sum + dram__bytes_write.sum of this kernel in a "
                                       "capture of the bench command (profiles/)") if dk["traffic"] else
                                      "null: no ncu capture of the current kernel build at this workload",
                    "note": "sparse outer products over coupling lists (4 n_b n_k FLOPs and 9 bytes per coupling; "
                            "coefficient rows gathered from L2): bound by the FP32 pipe, not by HBM or the tensor "
                            "cores; the HBM fraction is given beside it"}
    else:
        roofline = None

    variants = {}
    if not args.no_variants and world == 1:
        fp64_steps = 3 if args.config == 3 else max(2, args.steps // 2)
        for prec in ("fp64", "bf16x3", "tf32x3"):
            if prec == args.precision:
                variants[prec] = {"s_per_iter": s_per_iter, "E_first": energies[0]}
                continue
            v, Es, _ = time_variant(sysd, prec, fp64_steps if prec == "fp64" else max(2, args.steps // 2),
                                    args.warmup, l2_flush)
            variants[prec] = {"s_per_iter": v}
        del it
        torch.cuda.empty_cache()
        it = None
        # accuracy at identical states: converged ground state of every variant from the initial states
        variants["accuracy"] = accuracy_check(sysd)
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        if args.config == 1:
            dt, e_cpu, parts = time_oracle(sysd)
            cpu = {"value": dt, "unit": "s/iter", "cores": cpu_threads(), "kind": "port",
                   "sample": "one full iteration (densities + H + dense eigensolve, no gradient) of the same "
                             "workload with the NumPy FP64 oracle, BLAS threads = all cores",
                   "parts_s": parts, "E0": e_cpu}
            acc = variants.get("accuracy")
            if acc:
                for prec, rec in acc.items():
                    rec["dE0_vs_oracle"] = abs(rec["E0"] - e_cpu)
        else:
            smp = oracle_sampled_iteration(sysd, h_flops_of(sysd, args.config))
            cpu = {"value": smp["total"], "unit": "s/iter", "cores": cpu_threads(), "kind": "port",
                   "extrapolated": True,
                   "sample": "NumPy FP64 oracle (the reference's algorithm) on a bounded sample, extrapolated: every "
                             "density block of one fragment on a random subset of ket configurations and 1-2 / 2-4 "
                             "bra states (linear in both), H build = its algorithmic FLOPs at the measured host BLAS "
                             "rate, dense eigensolve scaled by n^3 from n = 2000; no gradient (a lower bound)",
                   "parts_s": {k: smp[k] for k in ("densities", "h_build", "eigensolve")},
                   "blas_gflops": smp["blas_gflops"]}
    plan_info = h_entries_of(sysd, args.config)
    line = {
        "metric": METRIC, "value": s_per_iter, "unit": "s/iter", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": {"fp64": "f64"}.get(args.precision, args.precision),
        "data": "synthetic (seeded h ~ N(0,0.1), V = sum_K L L with K=40, Sz-definite QR-orthonormal Gaussian CI vectors)",
        "config": {"workload": workload_name(args), "precision": args.precision,
                   "l2": "flushed (256 MiB write) before every timed step", "parallelism": f"replicas x{world}",
                   "step": "one steepest-descent state-optimizer iteration: densities + XR-H build + FP64 Lanczos "
                           "ground state + adjoint state and orbital gradients + Loewdin step"},
        "e2e": {"value": e2e_s_per_iter, "unit": "s/iter", "h2d_bytes_per_step": h2d_bytes,
                "d2h_bytes_per_step": d2h_bytes},
        "gpu_launches": launches, "gpu_launches_per_iteration": per_iter, "roofline": roofline, "clocks": clocks,
        "h_entries_per_build": plan_info["entries"],
        "h_entries_per_s": plan_info["entries"] / s_per_iter,
        "energies": energies[:3], "lanczos_residual_last": residual_last, "flops_per_build": flops_per_build,
        "peaks_measured": live, "variants": variants,
    }
    if "fp64" in variants and args.precision != "fp64":
        line["speedup_vs_fp64_gpu"] = variants["fp64"]["s_per_iter"] / s_per_iter
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def h_entries_of(sysd, config):
    """Entries of the XR-H one build forms: the blocks of every total-charge sector (the
    blocks between different total charges vanish and are never formed)."""
    n = [{c: sysd["states"][m][c][0].shape[0] for c in sysd["charges"]} for m in range(2)]
    sectors = {}
    for c0, a in n[0].items():
        for c1, b in n[1].items():
            sectors[c0 + c1] = sectors.get(c0 + c1, 0) + a * b
    return {"entries": float(sum(d * d for d in sectors.values())), "sector_dims": sectors}


def h_flops_of(sysd, config=None):
    """Algorithmic FLOPs of one order-0 dimer H build in the reference's contraction order
    (host arithmetic only): for every charge block with equal total charges, every order-0
    label and every catalog permutation that the block's charge changes admit
    (diagrams/S{T,U,V}_diagrams.py), the precontraction once per cache key
    (precontract.py:80,86: label, fragments, charge pair) and the final contraction, each
    2 x the product of the extents of its indices; plus t00 / u000 (2 n^2 N^2 per monomer
    block).  The v0000 monomer term is counted with the density builds (monomer_2e)."""
    chg = list(sysd["charges"])
    n = [{c: sysd["states"][m][c][0].shape[0] for c in chg} for m in range(2)]
    N = 2 * sysd["n_orb"]
    # (Dchgs, permutations, precontraction index extents (beyond i, j), final extents (beyond ijkl))
    cat = {"t01": ((-1, +1), ((0, 1), (1, 0)), 2, 1), "u001": ((-1, +1), ((0, 1), (1, 0)), 2, 1),
           "u101": ((-1, +1), ((0, 1), (1, 0)), 2, 1), "u100": ((0, 0), ((0, 1), (1, 0)), 2, None),
           "v0101": ((0, 0), ((0, 1),), 4, 2), "v0001": ((-1, +1), ((0, 1), (1, 0)), 4, 1),
           "v0100": ((+1, -1), ((0, 1), (1, 0)), 4, 1), "v0011": ((-2, +2), ((0, 1), (1, 0)), 4, 2)}
    flops, seen = 0.0, set()
    for ci0 in chg:
        for ci1 in chg:
            for cj0 in chg:
                for cj1 in chg:
                    if ci0 + ci1 != cj0 + cj1:
                        continue
                    pairs = ((ci0, cj0), (ci1, cj1))
                    for lab, (dch, perms, pre_ext, fin_ext) in cat.items():
                        for perm in perms:
                            pc = tuple(pairs[k] for k in perm)
                            if not all(pc[k][0] - pc[k][1] == dch[k] for k in range(2)):
                                continue
                            A, B = perm
                            nai, naj = n[A][pc[0][0]], n[A][pc[0][1]]
                            nbi, nbj = n[B][pc[1][0]], n[B][pc[1][1]]
                            key = (lab, A, pc[0])
                            if key not in seen:
                                seen.add(key)
                                flops += 2.0 * nai * naj * N ** pre_ext
                            if fin_ext is not None:
                                flops += 2.0 * nai * naj * nbi * nbj * N ** fin_ext
    for m in range(2):
        for c in chg:
            flops += 2 * 2.0 * n[m][c] ** 2 * N ** 2          # t00 and u000
    return flops


def accuracy_check(sysd):
    """Every variant against FP64 at the initial states, with converged eigenpairs (restarted
    Lanczos to a residual of 1e-9): |dE0|, max |dH| over the sector matrices, and the relative
    errors of the tangent state gradient and of dE/dkappa."""
    import torch
    from qodeapplications_gb300 import synthetic as S
    from qodeapplications_gb300.autograd import XRDimerEnergy
    from qodeapplications_gb300.gradients import tangent_project
    chg = list(sysd["charges"])
    out, ref = {}, None
    sidx = S.spin_orbital_spatial_index([sysd["n_orb"]] * 2)
    for prec in ("fp64", "bf16x3", "tf32x3"):
        eng = XRDimerEnergy.from_system(sysd, precision=prec, tol=1e-9)
        h = torch.as_tensor(sysd["h"], device="cuda")
        V = torch.as_tensor(sysd["V"], device="cuda")
        z = [{c: torch.as_tensor(sysd["states"][m][c][0], device="cuda") for c in chg} for m in range(2)]
        E = float(eng(h, V, z))
        eng.adj.launch(eng.d_product)
        g = eng.adj.state_gradient()
        gt = torch.cat([tangent_project(g[m][c], z[m][c]).reshape(-1) for m in range(2) for c in chg])
        T = h.contiguous()
        kg = eng.adj.orbital_gradient(T, torch.zeros((2,) + T.shape, dtype=torch.float64, device="cuda"),
                                      V.contiguous(), sidx).clone()
        Hs = {t: sec["H"].clone() for t, sec in eng.plan.sectors.items()}
        rec = {"E0": E, "lanczos_residual": eng.residual}
        if ref is None:
            ref = (E, Hs, gt.clone(), kg)
        else:
            rec.update(dE0=abs(E - ref[0]), max_dH=max(float((Hs[t] - ref[1][t]).abs().max()) for t in Hs),
                       state_grad_rel=float((gt - ref[2]).norm() / ref[2].norm()),
                       orbital_grad_rel=float((kg - ref[3]).norm() / ref[3].norm()))
        out[prec] = rec
        del eng, Hs
        torch.cuda.empty_cache()
    return out


def run_trimer(args):
    """Linear trimer: one step = the three pair builds (densities, monomer and dimer blocks),
    the per-build trimer stage and restarted FP64 Lanczos (cycles of lanczos_m matrix-free
    H x v products, each cycle one CUDA graph) in the neutral sector until the lowest Ritz
    pair's residual is below 1e-6 -> converged lowest eigenvalue.  Variants: fp64 (pair builds and H x v in FP64)
    and the split form (3xTF32 pair builds, FP32-product / FP64-sum H x v)."""
    import torch
    import numpy as np
    from qodeapplications_gb300 import _lib
    from qodeapplications_gb300 import synthetic as S
    from qodeapplications_gb300.densities import FragmentSpace
    from qodeapplications_gb300.hamiltonian import DeviceIntegrals
    from qodeapplications_gb300.trimer_hv import XRTrimerHamiltonian
    if int(os.environ.get("RANK", "0")) != 0:
        return                       # one trimer on one GPU: under torchrun rank 0 alone runs it
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    c = dict(CONFIGS[2])
    if args.states:
        c["n_states"] = args.states
        c["name"] = c["name"].replace("40 states", f"{args.states} states").replace("(448 000 states)", "")
    charges = [+1, 0, -1]
    sysd = S.make_system(n_frag=3, n_orb=c["n_orb"], n_states=c["n_states"], charges=charges, seed=SEED)
    spaces = [FragmentSpace({q: sysd["states"][m][q][1] for q in charges}, c["n_orb"], 0, sysd["n_elec_ref"])
              for m in range(3)]
    ns = [{q: c["n_states"] for q in charges}] * 3
    ints = DeviceIntegrals(h=sysd["h"], V=sysd["V"], Ns=sysd["Ns"])
    host = [{q: torch.as_tensor(sysd["states"][m][q][0]).pin_memory() for q in charges} for m in range(3)]
    dev = [{q: t.to("cuda") for q, t in d.items()} for d in host]
    lanczos_m = 40
    lanczos_tol = 1e-6          # residual of the lowest Ritz pair, relative to max(1, |E0|)
    forms = {"fp64": ("fp64", "fp64"), "fp32": ("tf32x3", "fp32"), "tf32x3": ("tf32x3", "tf32x3"),
             "bf16x3": ("bf16x3", "bf16x3")}
    head = args.precision if args.precision in forms else "tf32x3"
    want = [head] if args.no_variants else [head] + [f for f in ("fp64", "fp32", "tf32x3") if f != head]
    out = {}
    for form in want:
        prec, hvp = forms[form]
        ham = XRTrimerHamiltonian(spaces, ns, [charges] * 3, ints, precision=prec, hv_precision=hvp, total_charge=0)
        ham.set_coeffs(dev)

        v_start = None

        def step():
            # every step: the pair builds and the trimer stage, then restarted Lanczos (the
            # Krylov loop replayed as one CUDA graph) from the same start vector until the
            # residual of the ground state is below lanczos_tol
            ham.build()
            if v_start is not None:
                ham.lanczos.v0.copy_(v_start)
            w, resid = ham.lowest(k=1, m=lanczos_m, tol=lanczos_tol, graph=True)
            return float(w[0]), float(resid)

        ham.build()
        ham.lowest(k=1, m=lanczos_m, graph=True)       # capture the Krylov graph, fix the start vector
        v_start = ham.lanczos.v0.clone()

        for _ in range(max(args.warmup, 3) if form == head else 1):
            step()
        torch.cuda.synchronize()
        n_steps = args.steps if form == head else max(1, min(args.steps, 2))
        _lib.LaunchCounter.count = 0
        ms, Es = [], []
        clock_path = os.path.join(tempfile.gettempdir(), f"xrh_clocks_t_{os.getpid()}.csv")
        with ClockSampler(clock_path) as cs:
            torch.cuda.nvtx.range_push("xrh_timed")
            for _ in range(n_steps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                Es.append(step())
                e1.record()
                torch.cuda.synchronize()
                ms.append(e0.elapsed_time(e1))
            torch.cuda.nvtx.range_pop()
        rec = {"s_per_iter": sum(ms) / 1e3 / n_steps, "E0": Es[-1][0], "resid": Es[-1][1],
               "gpu_launches": _lib.LaunchCounter.count, "clocks": cs.summary(int(os.environ.get("LOCAL_RANK", "0")))}
        # dominant kernel: stage B of H x v (x' segments, 2 n^4 N^2 FLOPs per trimer block)
        st = ham.stage_b
        st.run()
        torch.cuda.synchronize()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for _ in range(5):
            st.run()
        t1.record()
        torch.cuda.synchronize()
        rec["stageB_ms"] = t0.elapsed_time(t1) / 5
        rec["stageB_tflops"] = st.flops / (rec["stageB_ms"] * 1e-3) / 1e12
        rec["hv_gflop"] = ham.flops_apply / 1e9
        if form == head:
            # e2e: coefficients from pinned host memory in, the energy out, every step
            e2e = []
            for _ in range(n_steps):
                t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                t0.record()
                for m in range(3):
                    for q in charges:
                        dev[m][q].copy_(host[m][q], non_blocking=True)
                ham.set_coeffs(dev)
                step()
                t1.record()
                torch.cuda.synchronize()
                e2e.append(t0.elapsed_time(t1))
            rec["e2e"] = sum(e2e) / 1e3 / n_steps
            rec["h2d"] = sum(t.numel() * 8 for d in host for t in d.values())
        out[form] = rec
        del ham
        torch.cuda.empty_cache()
    r = out[head]
    peaks = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(HERE, "MEASURED_PEAKS.json")) else {}
    peak = float(peaks.get("bf16_tflops", 1900.0)) if head in ("tf32x3", "bf16x3") else None
    line = {
        "metric": "XR-H trimer build + matrix-free Lanczos ground state s/iter", "value": r["s_per_iter"],
        "unit": "s/iter", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": r["s_per_iter"] * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": {"fp64": "f64", "fp32": "tf32x3 pair builds, fp32-product H x v"}.get(
            head, f"{head} (pair builds and the dominant H x v stage on tcgen05)"),
        "data": "synthetic (seeded h ~ N(0,0.1), V = sum_K L L with K=40, Sz-definite QR-orthonormal Gaussian CI vectors)",
        "config": {"workload": c["name"], "lanczos_steps_per_cycle": lanczos_m, "lanczos_residual_tol": lanczos_tol,
                   "l2": "inputs larger than L2 (pair sector matrices and intermediates of several GB)",
                   "step": "three pair builds + trimer stage 1 + restarted FP64 Lanczos on H x v to a ground-state "
                           "residual of 1e-6 (cycles of 40 steps replayed as CUDA graphs)"},
        "e2e": {"value": r["e2e"], "unit": "s/iter", "h2d_bytes_per_step": r["h2d"], "d2h_bytes_per_step": 8},
        "gpu_launches": r["gpu_launches"], "clocks": r["clocks"], "E0": r["E0"], "resid": r["resid"],
        "roofline": {"bound": {"fp64": "fp64 pipe", "fp32": "fp32 pipe"}.get(head, "tensor"),
                     "kernel": "H x v stage B (" + ("gemm_tc_kernel" if head in ("tf32x3", "bf16x3") else "gemm_fp64_kernel") + ")",
                     "achieved": r["stageB_tflops"], "unit": "TFLOP/s", "launch_ms": r["stageB_ms"],
                     "peak": peak, "frac": (r["stageB_tflops"] / peak) if peak else None, "traffic": None,
                     "note": "achieved = algorithmic FLOPs (2 n^4 N^2 per trimer block) / CUDA-event time of the "
                             "launch; tensor forms issue 3 MMAs per algorithmic FLOP and TF32 runs at half the BF16 "
                             "rate, peak = MEASURED_PEAKS.json bf16_tflops (of measured); no FP64/FP32 peak is "
                             "measured, so the SIMT forms carry none"},
        "variants": out,
    }
    if "fp64" in out:
        for f, rec in out.items():
            if f != "fp64":
                rec["dE0_vs_fp64"] = abs(rec["E0"] - out["fp64"]["E0"])
                rec["speedup_vs_fp64"] = out["fp64"]["s_per_iter"] / rec["s_per_iter"]
        if head != "fp64":
            line["speedup_vs_fp64_gpu"] = out[head]["speedup_vs_fp64"]
    print(json.dumps(line))


def run_ring(args):
    """Ring of 8 fragments: one step = every pair (densities, neutral-sector build, converged
    FP64 Lanczos, reverse pass into the state gradient of the pair expansion E2), the monomer
    terms, and every nearest-neighbour triple (densities, pair sectors, trimer stage,
    restarted matrix-free Lanczos with the Krylov loop as a CUDA graph), each ground state
    from the same fixed start vector to a residual of 1e-6.  Variant: the FP64 pair phase
    (E2 and its gradient) for the accuracy and speed of the split form."""
    import torch
    from qodeapplications_gb300 import _lib
    from qodeapplications_gb300.ring import XRRing
    if int(os.environ.get("RANK", "0")) != 0:
        return                       # one ring on one GPU: under torchrun rank 0 alone runs it
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    c = dict(CONFIGS[4])
    n_states = args.states or c["n_states"]
    n_orb = args.orbitals or c["n_orb"]
    name = c["name"]
    if args.states or args.orbitals:
        name = (f"ring of 8 fragments x {n_orb} spatial orbitals ({2 * n_orb} spin orbitals each), {n_states} "
                "states per charge sector (+1,0,-1): all 28 pairs (neutral sectors) and the 8 nearest-neighbour "
                "triples (neutral sectors)")
    triples = not args.no_triples
    if not triples:
        name = name.split(" and the 8 nearest")[0].replace("all 28 pairs", "all 28 pairs and the monomers")
    head = args.precision if args.precision in ("tf32x3", "bf16x3", "fp64") else "tf32x3"
    tol = 1e-6

    def log(msg):
        print(msg, file=sys.stderr, flush=True)

    t_setup = time.time()
    ring = XRRing(n_frag=c["n_frag"], n_orb=n_orb, n_states=n_states, precision=head, triples=triples, tol=tol,
                  seed=SEED)
    log(f"ring set up in {time.time() - t_setup:.1f} s, {torch.cuda.max_memory_allocated() / 1e9:.1f} GB allocated")
    host = [{q: z.cpu().pin_memory() for q, z in zf.items()} for zf in ring.coeffs]
    for _ in range(max(args.warmup, 3)):
        t0 = time.time()
        ring.iterate()
        log(f"warm-up iteration {time.time() - t0:.1f} s  phases {ring.phase_ms}")
    ring.check_status()
    torch.cuda.synchronize()
    _lib.LaunchCounter.count = 0
    ms, outs, phases = [], [], []
    clock_path = os.path.join(tempfile.gettempdir(), f"xrh_clocks_r_{os.getpid()}.csv")
    with ClockSampler(clock_path) as cs:
        torch.cuda.nvtx.range_push("xrh_timed")
        for _ in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            outs.append(ring.iterate())
            e1.record()
            torch.cuda.synchronize()
            ms.append(e0.elapsed_time(e1))
            phases.append(dict(ring.phase_ms))
        torch.cuda.nvtx.range_pop()
    launches = _lib.LaunchCounter.count
    clocks = cs.summary(local)
    s_per_iter = sum(ms) / 1e3 / args.steps
    resid_max = max(ring.resid.values())
    g_split = [{q: g.clone() for q, g in gf.items()} for gf in ring.grad]
    # e2e: coefficients from pinned host memory in, the two energies out, every step
    e2e = []
    for _ in range(args.steps):
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for f, zf in enumerate(ring.coeffs):
            for q, z in zf.items():
                z.copy_(host[f][q], non_blocking=True)
        ring.iterate()
        t1.record()
        torch.cuda.synchronize()
        e2e.append(t0.elapsed_time(t1))
    h2d = sum(t.numel() * 8 for d in host for t in d.values())
    # dominant kernel: stage B of the triples' H x v (or the density adjoint without triples)
    roof = None
    if triples and head != "fp64":
        st = ring.slot.stage_b
        st.run()
        torch.cuda.synchronize()
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        for _ in range(5):
            st.run()
        t1.record()
        torch.cuda.synchronize()
        sb_ms = t0.elapsed_time(t1) / 5
        peaks = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json"))) if os.path.exists(
            os.path.join(HERE, "MEASURED_PEAKS.json")) else {}
        peak = float(peaks.get("bf16_tflops", 1900.0))
        tfl = st.flops / (sb_ms * 1e-3) / 1e12
        roof = {"bound": "tensor", "kernel": "triple H x v stage B (gemm_tc_kernel)", "achieved": tfl,
                "unit": "TFLOP/s", "launch_ms": sb_ms, "flops_per_launch": st.flops, "peak": peak,
                "frac": tfl / peak, "traffic": None,
                "note": "achieved = algorithmic FLOPs (2 n^4 N^2 per trimer block) / CUDA-event time of the launch; "
                        "split forms issue 3 MMAs per algorithmic FLOP; peak = MEASURED_PEAKS.json bf16_tflops "
                        "(of measured)",
                "hv_gflop": ring.slot.flops_apply / 1e9}
    rec = {"s_per_iter": s_per_iter, "E2": outs[-1]["E2"], "E3": outs[-1]["E3"], "phases_ms": phases[-1],
           "max_lanczos_residual": resid_max, "n_pairs": len(ring.pairs), "n_triples": len(ring.triples),
           "triple_hv_products": sum(ring.products.values())}
    E_pair, E_mono = dict(ring.E_pair), dict(ring.E_mono)
    variants = {head: rec}
    triple_products = sum(ring.products.values())
    del ring
    torch.cuda.empty_cache()
    if not args.no_variants and head != "fp64":
        # FP64: the pair phase (E2 and its gradient) in full, one iteration; the triple phase from
        # one triple's FP64 build and H x v products timed, times the split run's product count
        r64 = XRRing(n_frag=c["n_frag"], n_orb=n_orb, n_states=n_states, precision="fp64", triples=triples,
                     tol=tol, seed=SEED)
        t0, t1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        t0.record()
        o64 = r64.iterate(with_triples=False)
        t1.record()
        torch.cuda.synchronize()
        num = den = 0.0
        for f in range(len(g_split)):
            for q in g_split[f]:
                num += float((r64.grad[f][q] - g_split[f][q]).norm()) ** 2
                den += float(r64.grad[f][q].norm()) ** 2
        v64 = {"s_per_iter_pairs": t0.elapsed_time(t1) / 1e3, "E2": o64["E2"],
               "max_lanczos_residual": max(r64.resid.values())}
        rec["dE2_vs_fp64"] = abs(rec["E2"] - o64["E2"])
        rec["max_pair_dE_vs_fp64"] = max(abs(E_pair[p] - r64.E_pair[p]) for p in E_pair)
        rec["max_monomer_dE_vs_fp64"] = max(abs(E_mono[f] - r64.E_mono[f]) for f in E_mono)
        rec["state_grad_rel_vs_fp64"] = (num / den) ** 0.5 if den > 0 else None
        rec["pairs_speedup_vs_fp64"] = v64["s_per_iter_pairs"] / (rec["phases_ms"]["pairs"] / 1e3)
        if triples:
            from qodeapplications_gb300.trimer_hv import PAIRS as _P
            T = r64.triples[0]
            S_ = r64.slot
            S_.set_coeffs([r64.coeffs[f] for f in T])
            S_.load_integral_sets([r64.pair_sets[(T[a], T[b])] for a, b in _P], r64.triple_sets[T])
            x = torch.ones(S_.dim, dtype=torch.float64, device="cuda") / S_.dim ** 0.5
            S_.build()
            S_.apply(x)
            e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
            e[0].record()
            S_.build()
            e[1].record()
            for _ in range(2):
                S_.apply(x)
            e[2].record()
            torch.cuda.synchronize()
            build_s, hv_s = e[0].elapsed_time(e[1]) / 1e3, e[1].elapsed_time(e[2]) / 2e3
            v64["triple_build_s"], v64["triple_hv_s"] = build_s, hv_s
            v64["triples_s_extrapolated"] = len(r64.triples) * build_s + triple_products * hv_s
            v64["s_per_iter_extrapolated"] = v64["s_per_iter_pairs"] + v64["triples_s_extrapolated"]
            v64["extrapolation"] = ("FP64 pair phase measured in full; FP64 triple phase = 8 FP64 triple builds + "
                                    "the split run's H x v product count x one FP64 product, each timed on triple "
                                    f"{T}; the FP64 Lanczos of the triples is not run (about "
                                    f"{v64['triples_s_extrapolated'] / 60:.0f} min)")
            rec["speedup_vs_fp64_extrapolated"] = v64["s_per_iter_extrapolated"] / rec["s_per_iter"]
        variants["fp64"] = v64
        del r64
        torch.cuda.empty_cache()
    line = {
        "metric": "XR ring build + gradient s/iter (pair expansion E2 with its state gradient, nearest-neighbour "
                  "triple increments E3)",
        "value": s_per_iter, "unit": "s/iter", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": s_per_iter * 1e3, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if head == "fp64" else f"{head} (pair builds and triple H x v on tcgen05; FP64 Lanczos)",
        "data": "synthetic (seeded h ~ N(0,0.1), V = sum_K L L with K=40, Sz-definite QR-orthonormal Gaussian CI "
                "vectors), the ChainIntegralSource ring",
        "config": {"workload": name, "lanczos_residual_tol": tol,
                   "l2": "inputs larger than L2 (pair sector matrices of 7.2 GB, densities of several GB)",
                   "step": "28 pair builds + Lanczos + reverse passes, 8 monomer ground states, 8 triple builds + "
                           "restarted matrix-free Lanczos (Krylov cycles as CUDA graphs), every ground state started "
                           "from lower orders of the same step plus a fixed random vector"},
        "e2e": {"value": sum(e2e) / 1e3 / args.steps, "unit": "s/iter", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": 16},
        "gpu_launches": launches, "clocks": clocks, "E2": rec["E2"], "E3": rec["E3"], "roofline": roof,
        "variants": variants,
    }
    if "speedup_vs_fp64_extrapolated" in rec:
        line["speedup_vs_fp64_gpu"] = rec["speedup_vs_fp64_extrapolated"]
    print(json.dumps(line))


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if args.config == 2:
        print(json.dumps({"impl": "reference", "unavailable": "the reference diagonalises the dense three-fragment "
                          "H, 1.7 M x 1.7 M at this size (23 TB in FP64); no CPU run of it is possible"}))
        return
    if args.config == 4:
        print(json.dumps({"impl": "reference", "unavailable": "the reference forms the product-basis H of all eight "
                          "fragments (300^8 states); no CPU run of it is possible"}))
        return
    sysd = make_system(args.config, args.states, args.orbitals)
    times, extra = [], {}
    n_timed = min(args.steps, 2)      # each oracle iteration takes tens of seconds: keep the run to minutes
    for _ in range(n_timed):
        if args.config == 1:
            dt, e, parts = time_oracle(sysd)
            extra = {"E0": e, "parts_s": parts}
            sample = (f"{n_timed} full iteration(s) of the workload (densities + H + dense eigensolve, no "
                      "gradient) with the NumPy FP64 oracle (restatement of the reference; the reference's own "
                      "Python path needs Qode)")
        else:
            smp = oracle_sampled_iteration(sysd, h_flops_of(sysd))
            dt = smp["total"]
            extra = {"extrapolated": True, "parts_s": {k: smp[k] for k in ("densities", "h_build", "eigensolve")},
                     "blas_gflops": smp["blas_gflops"]}
            sample = (f"{n_timed} bounded sample(s) of the workload with the NumPy FP64 oracle, extrapolated to the "
                      "full size: every density block on a random subset of ket configurations and 1-4 bra states, "
                      "H build = its algorithmic FLOPs at the measured host BLAS rate, dense eigensolve scaled by "
                      "n^3; no gradient (a lower bound of a reference iteration)")
        times.append(dt)
    v = sum(times) / len(times)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "s/iter", "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (same seeded system)",
            "config": {"workload": workload_name(args), "step": "densities + H build + FP64 eigensolve"},
            "cpu_baseline": dict({"value": v, "unit": "s/iter", "cores": cpu_threads(), "kind": "port",
                                  "sample": sample}, **extra),
            "e2e": {"value": v, "unit": "s/iter", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.config == 2:
        run_trimer(a)
    elif a.config == 4:
        run_ring(a)
    else:
        run_ours(a)

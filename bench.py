#!/usr/bin/env python
"""Benchmark: excitonic-Hamiltonian build (+ gradient) seconds per optimizer iteration.

One step = one optimizer iteration of the state optimisation on a seeded synthetic dimer:
transition densities of both fragments from the current states, the order-0 XR-H build,
its lowest eigenpair (FP64), and the energy gradient (state coefficients and orbital
rotations) when the adjoint is enabled.  `value` is device-resident (inputs in HBM);
`e2e` goes through the same public API with the states in pinned host memory and the
energy/gradient copied back every step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--config 1|3] [--precision P]
  python bench.py --impl reference ...   (the FP64 CPU oracle on the host cores)

Multi-GPU: the path does not shard (one dimer), so N>1 runs N independent replicas
(one per rank, launched by torchrun); value = total iterations / max time over ranks.
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
    1: dict(n_orb=9, n_states=10, name="dimer 2x9 spatial orbitals (18 spin orbitals each), 10 states per charge "
                                      "sector (+1,0,-1; 3/4/5 electrons), order-0 XR-H 900x900"),
    3: dict(n_orb=14, n_states=60, name="dimer 2x14 spatial orbitals (28 spin orbitals each), 60 states per charge "
                                       "sector (+1,0,-1), order-0 XR-H 32400x32400"),
}
SEED = 1234
METRIC = "XR-H build+grad s/iter vs plain FP64 GPU, at |dE|<=1e-6 Eh vs FP64 oracle"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--config", type=int, default=1, choices=sorted(CONFIGS))
    p.add_argument("--precision", default="fp64")
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


def make_system(cfg):
    from qodeapplications_gb300 import synthetic as S
    c = CONFIGS[cfg]
    return S.make_system(n_frag=2, n_orb=c["n_orb"], n_states=c["n_states"], charges=(+1, 0, -1), seed=SEED)


# ------------------------------------------------------------------------------------------
# CPU oracle step (reference arm and cpu_baseline)
# ------------------------------------------------------------------------------------------

def oracle_step(sysd):
    sys.path.insert(0, os.path.join(HERE, "oracle"))
    import numpy as np
    import xr_oracle as O
    charges = list(sysd["charges"])
    ints = O.FragInts(sysd["h"], sysd["V"], sysd["Ns"])
    dens = [O.build_densities({c: O.Sector(*sysd["states"][m][c]) for c in charges}, sysd["n_orb"],
                              sysd["n_core"], sysd["n_elec_ref"]) for m in range(2)]
    H1, H2 = O.get_xr_H0(ints, dens, [charges, charges])
    H = O.full_H(H1, H2)
    w, v = np.linalg.eigh(H)
    return float(w[0])


def time_oracle(sysd, budget_s=30.0):
    t0 = time.perf_counter()
    e = oracle_step(sysd)
    dt = time.perf_counter() - t0
    return dt, e


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
    """Device-resident optimizer iteration: densities -> H -> lowest eigenpair."""

    def __init__(self, sysd, precision):
        import torch
        from qodeapplications_gb300.densities import FragmentSpace
        from qodeapplications_gb300.hamiltonian import DeviceIntegrals, XRDimerPlan
        self.torch = torch
        charges = list(sysd["charges"])
        self.charges = charges
        spaces = [FragmentSpace({c: sysd["states"][m][c][1] for c in charges}, sysd["n_orb"], sysd["n_core"],
                                sysd["n_elec_ref"]) for m in range(2)]
        ns = [{c: sysd["states"][m][c][0].shape[0] for c in charges} for m in range(2)]
        self.plan = XRDimerPlan(spaces, ns, [charges, charges], DeviceIntegrals(h=sysd["h"], V=sysd["V"], Ns=sysd["Ns"]),
                                output="full", precision=precision)
        self.coeffs = [{c: torch.as_tensor(sysd["states"][m][c][0], device="cuda").contiguous() for c in charges}
                       for m in range(2)]
        self.host = [{c: torch.as_tensor(sysd["states"][m][c][0]).pin_memory() for c in charges} for m in range(2)]
        self.h2d_bytes = sum(t.numel() * 8 for d in self.host for t in d.values())
        self.E_host = torch.empty(1, dtype=torch.float64).pin_memory()
        self.phase_events = []

    def step(self, events=None):
        torch = self.torch
        if events is not None:
            events[0].record()
        for m in (0, 1):
            self.plan.builders[m].build(self.coeffs[m])
        for m in (0, 1):
            for c, sg in self.plan.sigma[m].items():
                sg.zrow.copy_(self.coeffs[m][c])
                sg.run_sigma(self.plan.builders[m].zT[c])
                self.plan.H1blk[m][c].zero_()
                self.plan.DU[m][c].zero_()
                self.plan.FULLD[m][c].zero_()
        if events is not None:
            events[1].record()
        self.plan.pre.run()
        if events is not None:
            events[2].record()
        self.plan.fin.run()
        if events is not None:
            events[3].record()
        w, v = torch.linalg.eigh(self.plan.H)
        if events is not None:
            events[4].record()
        return w[:1]

    def step_e2e(self):
        for m in (0, 1):
            for c in self.charges:
                self.coeffs[m][c].copy_(self.host[m][c], non_blocking=True)
        e = self.step()
        self.E_host.copy_(e, non_blocking=True)
        return self.E_host


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
    sysd = make_system(args.config)
    it = GPUIteration(sysd, args.precision)
    l2_flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    for _ in range(max(args.warmup, 3)):
        it.step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    clock_path = os.path.join(tempfile.gettempdir(), f"xrh_clocks_{os.getpid()}.csv")
    n_ph = 5
    step_ms, phase_ms = [], [0.0] * (n_ph - 1)
    barrier()
    _lib.LaunchCounter.count = 0
    with ClockSampler(clock_path) as cs:
        for _ in range(args.steps):
            l2_flush.zero_()
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(n_ph)]
            it.step(ev)
            torch.cuda.synchronize()
            step_ms.append(ev[0].elapsed_time(ev[-1]))
            for k in range(n_ph - 1):
                phase_ms[k] += ev[k].elapsed_time(ev[k + 1])
        barrier()
    launches = _lib.LaunchCounter.count
    clocks = cs.summary(local)
    total_ms = sum(step_ms)

    # end-to-end through host buffers
    barrier()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record()
    for _ in range(args.steps):
        it.step_e2e()
    t1.record()
    torch.cuda.synchronize()
    e2e_ms = t0.elapsed_time(t1)
    E0 = float(it.E_host[0])

    tens = torch.tensor([total_ms, e2e_ms], device="cuda")
    if world > 1:
        dist.all_reduce(tens, op=dist.ReduceOp.MAX)
    total_ms, e2e_ms = float(tens[0]), float(tens[1])
    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return

    s_per_iter = total_ms / 1e3 / args.steps
    # roofline of the dominant kernel launch (by measured phase time)
    names = ["densities+sigma", "precontraction GEMM", "final GEMM", "eigensolve"]
    phases = {n: phase_ms[k] / args.steps for k, n in enumerate(names)}
    flops_fin = it.plan.fin.flops
    fin_ms = phases["final GEMM"]
    peaks = json.load(open(os.path.join(HERE, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(HERE, "MEASURED_PEAKS.json")) else {}
    fp64_peak = measure_fp64_peak()
    roofline = {"bound": "tensor", "kernel": "gemm_fp64_kernel (final, grouped)", "achieved": flops_fin / (fin_ms * 1e-3) / 1e12,
                "peak": fp64_peak, "unit": "TFLOP/s", "frac": (flops_fin / (fin_ms * 1e-3) / 1e12) / fp64_peak,
                "peak_source": "FP64 DGEMM (torch.matmul float64 8192^3) measured in this run; MEASURED_PEAKS.json has no FP64 figure",
                "traffic": None}
    cpu = None
    if not args.no_cpu_baseline and world == 1:
        dt, e_cpu = time_oracle(sysd)
        cpu = {"value": dt, "unit": "s/iter", "cores": os.cpu_count(), "kind": "port",
               "sample": "one full iteration of the same workload with the NumPy FP64 oracle (BLAS threads = all cores)",
               "E0": e_cpu, "dE_gpu_vs_oracle": abs(e_cpu - E0)}
    line = {
        "metric": METRIC, "value": s_per_iter, "unit": "s/iter", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else args.precision,
        "data": "synthetic (seeded h ~ N(0,0.1), V = sum_K L L with K=40, Sz-definite QR-orthonormal Gaussian CI vectors)",
        "config": {"workload": CONFIGS[args.config]["name"], "precision": args.precision,
                   "l2": "flushed (256 MiB write) before every timed step", "parallelism": f"replicas x{world}",
                   "step": "densities + H build + FP64 eigensolve"},
        "e2e": {"value": e2e_ms / 1e3 / args.steps, "unit": "s/iter", "h2d_bytes_per_step": it.h2d_bytes,
                "d2h_bytes_per_step": 8},
        "gpu_launches": launches, "phases_ms": phases, "roofline": roofline, "clocks": clocks,
        "E0": E0, "flops_per_iter": it.plan.flops, "peaks": {k: peaks.get(k) for k in ("hbm_gbs", "bf16_tflops")},
    }
    if cpu:
        line["cpu_baseline"] = cpu
    print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def measure_fp64_peak():
    import torch
    a = torch.randn(8192, 8192, dtype=torch.float64, device="cuda")
    b = torch.randn(8192, 8192, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(3):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.matmul(a, b)
        e.record()
        torch.cuda.synchronize()
        best = min(best, s.elapsed_time(e))
    return 2 * 8192 ** 3 / (best * 1e-3) / 1e12


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sysd = make_system(args.config)
    times = []
    n_timed = min(args.steps, 2)      # each oracle iteration takes tens of seconds: keep the run to minutes
    for _ in range(n_timed):
        dt, e = time_oracle(sysd)
        times.append(dt)
    v = sum(times) / len(times)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "s/iter", "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (same seeded system)",
            "config": {"workload": CONFIGS[args.config]["name"], "step": "densities + H build + FP64 eigensolve"},
            "cpu_baseline": {"value": v, "unit": "s/iter", "cores": os.cpu_count(), "kind": "port",
                             "sample": f"{n_timed} full iteration(s) of the workload with the NumPy FP64 oracle "
                                       "(restatement of the reference; the reference's own Python path needs Qode)"},
            "e2e": {"value": v, "unit": "s/iter", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}, "E0": e}
    print(json.dumps(line))


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)

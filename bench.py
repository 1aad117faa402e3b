"""Benchmark: 30-qubit, 40-layer random circuit (2260 gates incl. QFT) on one GB300.

Workload (the configuration the headline metric is quoted on): 2^30 complex
amplitudes, |+>^30 initial state, 40 layers of one random single-qubit gate
per qubit (H,X,Y,Z,S,T,RX,RY,RZ,P; seed 0) plus a CNOT brickwork, then the
QFT on all 30 qubits.  Synthetic, seeded data (no dataset is involved).

One step = one execution of the whole circuit on the resident state
(state reset to |+>^30, then the fused complex-FP32 plan).  The metric is
layers/s (40 layers per step).  Inputs (8 GiB of FP32 amplitudes) are far
larger than the 129 MB L2, so no L2 flush is needed between steps.

Besides the JSON keys the contract requires, the line carries the plain FP64
per-gate CUDA path (the >= 8x target's denominator), the complex-FP32
per-gate path, and the fused path's infidelity against the FP64 per-gate
result (FP64 accumulation on the device).

--impl reference times the reference implementation's CPU data flow (the
oracle port of the rayon branch, oracle/qi_oracle.cpp) on a bounded sample.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_QUBITS = 30
LAYERS = 40
SEED = 0
FUSED_K = 6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--qubits", type=int, default=N_QUBITS)
    ap.add_argument("--skip-baselines", action="store_true", help="skip FP64/FP32 per-gate and CPU legs")
    ap.add_argument("--profile-case", default=None, choices=["fused26", "trotter26", "adjoint26"],
                    help="run a small fixed case for ncu captures instead of the benchmark")
    return ap.parse_args()


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.path = os.environ.get("QI_BENCH_CLOCKS_CSV",
                                   os.path.join(tempfile.gettempdir(), "qi_bench_clocks_%d.csv" % os.getpid()))

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_port_sample(n, gates, budget_gates, threads):
    """Time the oracle port of the reference's rayon data flow on the first
    `budget_gates` gates at n qubits; returns (seconds per gate, gates timed, n)."""
    import numpy as np
    from oracle import oracle as orc
    from quant_iron_gb300 import workloads
    init = workloads.plus_state(n)
    _, secs = orc.port_execute(init, n, gates[:budget_gates], threads)
    del init
    return secs / budget_gates


def replica_throughput(ms, world, steps, device="cuda"):
    """Whole-job throughput of `world` replicas: each rank processed LAYERS x steps layers
    in its own ms; the job took the slowest rank's time (all_reduce MAX)."""
    if world > 1:
        import torch
        import torch.distributed as dist
        t = torch.tensor([ms], dtype=torch.float64, device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * LAYERS * steps / (ms / 1e3)


def host_mem_gb():
    try:
        for line in open("/proc/meminfo"):
            if line.startswith("MemAvailable:"):
                return int(line.split()[1]) / 1e6
    except Exception:
        pass
    return 0.0


def cpu_baseline(n, gates, budget_s=25.0):
    """Bounded sample of the reference CPU data flow; picks the gate count to stay near budget_s."""
    threads = os.cpu_count() or 1
    # the rayon data flow holds ~56 B/amp (state, clone, update list); fall back to fewer qubits if short
    need_gb = (1 << n) * 60 / 1e9
    nn = n
    while nn > 20 and host_mem_gb() < need_gb * 1.3:
        nn -= 1
        need_gb = (1 << nn) * 60 / 1e9
    from quant_iron_gb300 import workloads
    g = gates if nn == n else workloads.random_circuit(nn, LAYERS, seed=SEED)
    t1 = cpu_port_sample(nn, g, 1, threads)
    k = max(1, min(len(g) - 1, int(budget_s / max(t1, 1e-6)) - 1))
    tk = cpu_port_sample(nn, g[1:], k, threads) if k > 0 else t1
    per_gate = tk * (1 << (n - nn))   # scale a smaller sample to n qubits by amplitude count
    step_s = per_gate * len(gates)
    return {"value": LAYERS / step_s, "unit": "layers/s", "cores": threads, "kind": "port",
            "sample": "oracle port of the reference rayon data flow (clone + per-pair update list + serial "
                      "scatter): %d gates of the %d-qubit circuit timed, extrapolated to all %d gates%s" %
                      (k + 1, nn, len(gates), "" if nn == n else " and scaled by 2^%d amplitudes" % (n - nn)),
            "seconds_per_gate": per_gate}


def adjoint_leg(qi, workloads, stream, torch, np, n=26, layers=12):
    """Adjoint gradient of the 26-qubit hardware-efficient ansatz (12 layers of RY.RZ + CNOT
    ladder, 624 parameters, seed 1) on the periodic XXZ energy: gradients/s with an FP32
    state, agreement with the FP64-state adjoint, and FP64 central differences (eps 1e-4)
    on 8 seeded parameters."""
    gates, theta = workloads.hea_ansatz(n, layers, seed=1)
    terms = workloads.xxz_periodic(n, seed=1)
    s32 = qi.DeviceState(n, qi.F32)
    s32.set_stream(stream.cuda_stream)
    s32.set_zero()
    qi.adjoint_gradient(s32, gates, theta, terms)   # warm-up
    reps = 3
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        e32, g32 = qi.adjoint_gradient(s32, gates, theta, terms)
    torch.cuda.synchronize()
    t_adj = (time.perf_counter() - t0) / reps
    s32.close()
    s64 = qi.DeviceState(n, qi.F64)
    s64.set_stream(stream.cuda_stream)
    s64.set_zero()
    e64, g64 = qi.adjoint_gradient(s64, gates, theta, terms)
    rel32 = float(np.linalg.norm(g32 - g64) / np.linalg.norm(g64))
    # FP64 central differences with the plain per-gate FP64 path
    rng = np.random.default_rng(1)
    ids = rng.choice(theta.size, 8, replace=False)
    fd = []
    for j in ids:
        vals = []
        for sgn in (1, -1):
            th = theta.copy()
            th[j] += sgn * 1e-4
            s64.set_zero()
            qi.Plan(n, qi.F64, gates, theta=th, fusion=qi.FUSION_NONE).execute(s64)
            vals.append(qi.sumop_expectation(s64, terms).real)
        fd.append((vals[0] - vals[1]) / 2e-4)
    fd = np.array(fd)
    rel_fd = float(np.linalg.norm(g64[ids] - fd) / np.linalg.norm(fd))
    rel_fd32 = float(np.linalg.norm(g32[ids] - fd) / np.linalg.norm(fd))
    s64.close()
    return {"workload": "HEA %d qubits, %d layers, %d parameters, periodic XXZ (%d terms)" % (n, layers, theta.size,
                                                                                             len(terms)),
            "grad_per_s_fp32": 1.0 / t_adj, "seconds_per_grad_fp32": t_adj, "energy_fp32": e32, "energy_fp64": e64,
            "rel_err_fp32_vs_fp64_adjoint": rel32, "rel_err_fp64_adjoint_vs_fd_subset": rel_fd,
            "rel_err_fp32_adjoint_vs_fd_subset": rel_fd32, "fd_subset": [int(x) for x in ids]}


def trotter_leg(qi, workloads, stream, torch, np, rows=5, cols=6, steps=20, observe_every=10):
    """First-order Trotter evolution on the 5x6 open lattice (30 qubits): anisotropic
    Heisenberg (1.0 XX + 0.8 YY + 0.5 ZZ per bond, h_i Z_i), 177 terms, dt = 0.05, from a
    seeded basis state.  The FP32 fused step (one plan per step, <H> every 10 steps) is
    timed over `steps` steps; the FP64 step (grouped exponentials: one pass per run of
    terms whose X-masks lie in {0, X}, i.e. one per bond plus the field run) is timed
    over 2 steps, and <H> after 2 steps of both is compared."""
    n = rows * cols
    terms = workloads.lattice_xyz(rows, cols, seed=0)
    basis = int(np.random.default_rng(0).integers(0, 1 << n))
    out = {"workload": "5x6 lattice anisotropic Heisenberg, %d terms, dt 0.05, basis state %d" % (len(terms), basis),
           "steps": steps}
    s32 = qi.DeviceState(n, qi.F32)
    s32.set_stream(stream.cuda_stream)
    s32.set_basis(basis)
    qi.trotter_evolve(s32, terms, 0.05, 2)   # warm-up (plan build, first launches)
    e32_2 = qi.sumop_expectation(s32, terms).real
    s32.set_basis(basis)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e32 = qi.trotter_evolve(s32, terms, 0.05, steps, observable=terms, observe_every=observe_every)
    t32 = time.perf_counter() - t0
    s32.close()
    s64 = qi.DeviceState(n, qi.F64)
    s64.set_stream(stream.cuda_stream)
    s64.set_basis(basis)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    qi.trotter_evolve(s64, terms, 0.05, 2)
    t64_step = (time.perf_counter() - t0) / 2
    e64_2 = qi.sumop_expectation(s64, terms).real
    s64.close()
    out.update({"fp32_fused_ms_per_step": t32 * 1e3 / steps, "fp64_grouped_ms_per_step": t64_step * 1e3,
                "speedup_fp32_fused_vs_fp64_grouped": t64_step / (t32 / steps),
                "term_exponentials_per_s_fp32": len(terms) * steps / t32,
                "energies_fp32_every_%d" % observe_every: [complex(e).real for e in e32],
                "energy_after_2_steps_fp32_fused": e32_2, "energy_after_2_steps_fp64_grouped": e64_2,
                "energy_error_fp32_2_steps": abs(e32_2 - e64_2),
                "note": "FP32 timed region includes the <H> evaluations (every %d steps)" % observe_every})
    return out


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    sys.path.insert(0, ROOT)
    import __graft_entry__ as ge
    ge.build_oracle()
    ge.load_package()
    from quant_iron_gb300 import workloads
    n = args.qubits
    gates = workloads.random_circuit(n, LAYERS, seed=SEED)
    threads = os.cpu_count() or 1
    need_gb = (1 << n) * 60 / 1e9
    nn = n
    while nn > 20 and host_mem_gb() < need_gb * 1.3:
        nn -= 1
        need_gb = (1 << nn) * 60 / 1e9
    g = gates if nn == n else workloads.random_circuit(nn, LAYERS, seed=SEED)
    per_step_gates = 2
    for _ in range(args.warmup):
        cpu_port_sample(nn, g, 1, threads)
    times = []
    for s in range(args.steps):
        off = (s * per_step_gates) % (len(g) - per_step_gates)
        times.append(cpu_port_sample(nn, g[off:], per_step_gates, threads))
    per_gate = statistics.mean(times) * (1 << (n - nn))
    step_s = per_gate * len(gates)
    value = LAYERS / step_s
    sample = ("oracle port of the reference rayon data flow on %d host threads: %d gates of the %d-qubit circuit per "
              "step, extrapolated to all %d gates%s" % (threads, per_step_gates, nn, len(gates),
                                                       "" if nn == n else " and scaled by 2^%d" % (n - nn)))
    line = {"impl": "reference", "metric": "layers/s", "value": value, "unit": "layers/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_s * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": {"workload": "random circuit, %d qubits, %d layers + QFT (%d gates), seed %d" %
                                   (n, LAYERS, len(gates), SEED), "qubits": n, "layers": LAYERS},
            "cpu_baseline": {"value": value, "unit": "layers/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "layers/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def profile_case_fused26():
    """Small case for ncu (26 qubits FP32 = 512 MB, larger than L2): the fused k<=6 plan of
    the 26-qubit random circuit, twice (k_fused_tc, k_phase_poly, k_diagk launches), then one
    <H> of the 26-qubit open-chain Heisenberg (k_xgroup_expect_f32, k_diag_expect_f32)."""
    import __graft_entry__ as ge
    qi = ge.load_package()
    from quant_iron_gb300 import workloads
    n = 26
    gates = workloads.random_circuit(n, LAYERS, seed=SEED)
    plan = qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=FUSED_K)
    st = qi.DeviceState(n, qi.F32)
    st.set_plus()
    for _ in range(2):
        plan.execute(st)
    st.synchronize()
    e = qi.sumop_expectation(st, workloads.heisenberg_open_chain(n)).real
    print("profile case done, norm^2 = %.9f, <H> = %.9f" % (st.norm_sqr(), e))


def profile_case_trotter26():
    """Small case for ncu (26 qubits FP64 = 1 GB): two FP64 Trotter steps of the 2x13 lattice
    anisotropic Heisenberg (76 terms) as grouped exponentials (k_pauli_group_pair,
    k_pauli_group_diag), then the same two steps of an FP32 state (fused plan)."""
    import __graft_entry__ as ge
    qi = ge.load_package()
    from quant_iron_gb300 import workloads
    n = 26
    terms = workloads.lattice_xyz(2, 13, seed=0)
    for prec in (qi.F64, qi.F32):
        st = qi.DeviceState(n, prec)
        st.set_plus()
        qi.trotter_evolve(st, terms, 0.05, 2)
        st.synchronize()
        print("profile case done, precision %d, norm^2 = %.9f" % (prec, st.norm_sqr()))
        st.close()


def profile_case_adjoint26():
    """Small case for ncu (26 qubits FP32 = 512 MB per state): one adjoint gradient of the
    26-qubit hardware-efficient ansatz (12 layers, 624 parameters) on the periodic XXZ
    energy — forward plan, <H>, lambda = H psi, then the grouped reverse sweep
    (k_adjoint_multi, fused inverse plans of the CNOT ladders)."""
    import __graft_entry__ as ge
    qi = ge.load_package()
    from quant_iron_gb300 import workloads
    n = 26
    import numpy as np
    gates, theta = workloads.hea_ansatz(n, 12, seed=1)
    terms = workloads.xxz_periodic(n, seed=1)
    st = qi.DeviceState(n, qi.F32)
    st.set_zero()
    e, g = qi.adjoint_gradient(st, gates, theta, terms)
    st.synchronize()
    print("profile case done, E = %.9f, |grad| = %.9f" % (e, float(np.linalg.norm(g))))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
        return
    if args.profile_case == "fused26":
        profile_case_fused26()
        return
    if args.profile_case == "trotter26":
        profile_case_trotter26()
        return
    if args.profile_case == "adjoint26":
        profile_case_adjoint26()
        return
    import numpy as np
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    import __graft_entry__ as ge
    ge.build()
    qi = ge.load_package()
    from quant_iron_gb300 import workloads
    qi._abi.check(qi._abi.lib.qi_set_device(local))

    n = args.qubits
    gates = workloads.random_circuit(n, LAYERS, seed=SEED)
    terms = workloads.heisenberg_open_chain(n, seed=SEED)
    t0 = time.perf_counter()
    plan = qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=FUSED_K)
    plan_s = time.perf_counter() - t0
    stats = plan.stats()
    stream = torch.cuda.Stream()
    st = qi.DeviceState(n, qi.F32)
    st.set_stream(stream.cuda_stream)

    def step():
        st.set_plus()
        plan.execute(st)

    def barrier():
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()

    for _ in range(args.warmup):
        step()
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    l0 = qi.launch_count()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    with torch.cuda.stream(stream):
        ev0.record(stream)
        for _ in range(args.steps):
            step()
        ev1.record(stream)
    barrier()
    launches = qi.launch_count() - l0
    clk = clocks.stop()
    ms, value = replica_throughput(ev0.elapsed_time(ev1), world, args.steps)
    ms_per_step = ms / args.steps

    # per-op device times of one execution (events on the launching stream)
    st.set_plus()
    ops, op_ms = qi.plan_profile(plan, st)
    by_kernel = {}
    for op, t in zip(ops, op_ms):
        name = qi.KERNEL_OF_OP_KIND.get(op["kind"], str(op["kind"]))
        if op["kind"] == 4:
            name = "k_fused_tc" if op.get("tensor_cores") else "k_fused_simt"
        d = by_kernel.setdefault(name, {"launches": 0, "ms": 0.0})
        d["launches"] += 1
        d["ms"] += t
    dom = max(by_kernel, key=lambda k: by_kernel[k]["ms"])
    peak, peak_kind = load_peaks()
    pass_bytes = (1 << n) * 8 * 2   # one read + one write of every FP32 amplitude
    avg_ms = by_kernel[dom]["ms"] / by_kernel[dom]["launches"]
    achieved = pass_bytes / (avg_ms / 1e3) / 1e9
    # DRAM traffic per launch from the committed ncu capture of a smaller case of the same kernel,
    # scaled by amplitude count (traffic grows in proportion to the state)
    traffic, traffic_src = None, None
    prof = os.path.join(ROOT, "profiles", "k_fused_tc_fused26_ncu.json")
    if dom == "k_fused_tc" and os.path.exists(prof):
        pj = json.load(open(prof))
        traffic = pj["traffic_per_amp_bytes"] * (1 << n)
        traffic_src = "profiles/k_fused_tc_fused26.md (26-qubit capture x 2^%d)" % (n - 26)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "traffic_source": traffic_src, "kernel": dom, "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": pass_bytes, "avg_launch_ms": avg_ms,
                "kernels": {k: {"launches": v["launches"], "ms": round(v["ms"], 3),
                                "share": round(v["ms"] / max(1e-9, sum(x["ms"] for x in by_kernel.values())), 4)}
                            for k, v in by_kernel.items()}}
    if dom == "k_fused_tc":
        # the same kernel against the tensor roof: 3 split products x 8 * 2^k flop per amplitude
        # (k = 6: 1536 flop/amp) per launch; peak = the nominal dense TF32 rate (no measured TF32
        # figure exists for this pool), so the fraction is of nominal
        tflop = 3 * 8 * (1 << FUSED_K) * (1 << n) / 1e12
        roofline["tensor"] = {"achieved": tflop / (avg_ms / 1e3), "peak": 1100.0, "unit": "TFLOP/s",
                              "frac": tflop / (avg_ms / 1e3) / 1100.0, "peak_source": "nominal dense TF32",
                              "flop_per_amp": 3 * 8 * (1 << FUSED_K)}

    # energy of the final state (FP64 reduction), and the time of SumOp::expectation_value
    energy = qi.sumop_expectation(st, terms).real
    ex_t = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        qi.sumop_expectation(st, terms)
        ex_t.append(time.perf_counter() - t0)
    n_groups = len({(int(t["xmask"])) for t in terms})
    expectation = {"terms": len(terms), "x_groups": n_groups, "ms": min(ex_t) * 1e3,
                   "passes_gbs": n_groups * (1 << n) * 8 / min(ex_t) / 1e9,
                   "note": "one read pass of the FP32 state per X-mask group, host call to result (synchronous)"}

    extra = {}
    if rank == 0 and not args.skip_baselines:
        # plain FP64 per-gate CUDA path (the denominator of the >= 8x target) and FP32 per-gate
        plan64 = qi.Plan(n, qi.F64, gates, fusion=qi.FUSION_NONE)
        s64 = qi.DeviceState(n, qi.F64)
        s64.set_stream(stream.cuda_stream)
        s64.set_plus()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plan64.execute(s64)
        e1.record(stream)
        torch.cuda.synchronize()
        ms64 = e0.elapsed_time(e1)
        energy64 = qi.sumop_expectation(s64, terms).real
        # infidelity of the fused FP32 result against the FP64 per-gate result
        st.set_plus()
        plan.execute(st)
        tmp = qi.DeviceState(n, qi.F32)
        tmp.set_stream(stream.cuda_stream)
        tmp.copy_from(s64)
        ov = tmp.inner_product(st)
        infid = 1.0 - abs(ov) ** 2 / (tmp.norm_sqr() * st.norm_sqr())
        # max amplitude error on a sampled stride of amplitudes
        idx = np.linspace(0, (1 << n) - 1, 4096).astype(np.int64)
        max_err = max(abs(st.amplitude(int(i)) - s64.amplitude(int(i))) for i in idx[:256])
        tmp.close()
        s64.close()
        del plan64
        plan32 = qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_NONE)
        st.set_plus()
        torch.cuda.synchronize()
        e0.record(stream)
        plan32.execute(st)
        e1.record(stream)
        torch.cuda.synchronize()
        ms32 = e0.elapsed_time(e1)
        del plan32
        extra = {"fp64_per_gate_ms": ms64, "fp32_per_gate_ms": ms32, "fused_fp32_ms": ms_per_step,
                 "speedup_fused_vs_fp64_per_gate": ms64 / ms_per_step,
                 "infidelity_fused_vs_fp64": infid, "max_amp_error_sampled": max_err,
                 "energy_fused_fp32": energy, "energy_fp64_per_gate": energy64,
                 "energy_error": abs(energy - energy64),
                 "gates_per_s_fused": len(gates) / (ms_per_step / 1e3)}
        extra["adjoint"] = adjoint_leg(qi, workloads, stream, torch, np)
        extra["trotter"] = trotter_leg(qi, workloads, stream, torch, np)
    extra["expectation"] = expectation

    # end-to-end through the public API with host buffers: H2D of the initial state,
    # the circuit, D2H of the final state, every step.  Two device states alternate:
    # each step's upload and download run on the copy engine (page-locked buffers,
    # qi_state_upload_async / download_async) while the other state's circuit runs.
    e2e = None
    if rank == 0:
        dim = 1 << n
        pipelined = host_mem_gb() > 3.5 * 16 * dim / 1e9
        host_in = torch.empty(2 * dim, dtype=torch.float64, pin_memory=True)
        host_in.fill_(1.0 / (dim ** 0.5))
        host_in[1::2] = 0.0
        if pipelined:
            host_out = [torch.empty(2 * dim, dtype=torch.float64, pin_memory=True) for _ in range(2)]
            stream2 = torch.cuda.Stream()
            st2 = qi.DeviceState(n, qi.F32)
            st2.set_stream(stream2.cuda_stream)
            states = [st, st2]
            for s2 in states:   # allocates each state's staging and second buffers (an allocation synchronises
                s2.upload_async(host_in.data_ptr(), dim)   # the device, so none may happen in the timed loop)
                plan.execute(s2)
                s2.synchronize()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        if pipelined:
            e2e_steps = max(2, args.steps)
            for k in range(e2e_steps):
                s2 = states[k % 2]
                s2.upload_async(host_in.data_ptr(), dim)
                plan.execute(s2)
                s2.download_async(host_out[k % 2].data_ptr(), dim)
            joined = torch.cuda.Event()
            joined.record(stream2)
            stream.wait_event(joined)
        else:   # not enough page-locked host memory for two output buffers: one state, in order
            e2e_steps = max(1, min(args.steps, 3))
            for _ in range(e2e_steps):
                st.upload_ptr(host_in.data_ptr(), dim)
                plan.execute(st)
                st.download_ptr(host_in.data_ptr(), dim)
        e1.record(stream)
        torch.cuda.synchronize()
        wall = time.perf_counter() - t0
        e2e_ms = e0.elapsed_time(e1)
        e2e = {"value": LAYERS * e2e_steps / (e2e_ms / 1e3), "unit": "layers/s", "h2d_bytes_per_step": 16 * dim,
               "d2h_bytes_per_step": 16 * dim, "wall_s": wall, "steps": e2e_steps,
               "pipeline": ("two device states; each step's H2D and D2H on the copy engine overlap the other "
                            "state's circuit" if pipelined else "one state, transfers in order")}
        if pipelined:
            st2.close()
            del host_out
        del host_in

    cpu = None
    if rank == 0 and world == 1 and not args.skip_baselines:
        st.close()
        cpu = cpu_baseline(n, gates)

    if rank == 0:
        line = {"metric": "layers/s", "value": value, "unit": "layers/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "c64", "data": "synthetic",
                "config": {"workload": "random circuit, %d qubits, %d layers + QFT (%d gates), |+>^%d, seed %d; "
                                       "fused complex-FP32 blocks k<=%d" % (n, LAYERS, len(gates), n, SEED, FUSED_K),
                           "qubits": n, "layers": LAYERS, "gates": len(gates), "fusion": "greedy k<=%d" % FUSED_K,
                           "plan": stats, "plan_build_s": plan_s,
                           "l2": "inputs (%d GiB state) larger than the 129 MB L2; no flush" % ((1 << n) * 8 >> 30),
                           "parallelism": "replicas" if world > 1 else "single GPU"},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk, "gpu_launches": launches}
        line.update(extra)
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()

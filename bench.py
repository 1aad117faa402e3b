"""Benchmark: 30-qubit, 40-layer random circuit (2260 gates incl. QFT) on one GB300.

Workload (the configuration the headline metric is quoted on): 2^30 complex
amplitudes, |+>^30 initial state, 40 layers of one random single-qubit gate
per qubit (H,X,Y,Z,S,T,RX,RY,RZ,P; seed 0) plus a CNOT brickwork, then the
QFT on all 30 qubits.  Synthetic, seeded data (no dataset is involved).

One step = one execution of the whole circuit on the resident state
(state reset to |+>^30, then the fused complex-FP32 plan).  The metric is
layers/s (40 layers per step).  Inputs (8 GiB of FP32 amplitudes) are far
larger than the 129 MB L2, so no L2 flush is needed between steps.

Besides the JSON keys the contract requires, the line carries the other
configurations of the workload family, each against an FP64 result on the device:
  seeds       the 30-qubit circuit on seeds 0-4: fused FP32 against the plain FP64
              per-gate path (the >= 8x target's denominator), infidelity, full-state
              max amplitude error, energy error, both times;
  per_gate    one kernel per gate by kind and target qubit, FP32 and FP64, as a
              fraction of the measured copy bandwidth;
  adjoint     26-qubit hardware-efficient ansatz gradient (624 parameters): FP32
              gradients/s, FP32 vs FP64 adjoint, FP64 central differences and
              parameter shift (seeded subsets; --adjoint-fd all for every parameter);
  trotter     100 first-order Trotter steps on the 5x6 lattice, Heisenberg and TFIM,
              FP32 fused vs FP64 grouped, <H> every 10 steps;
  e2e         the same circuit through the public API from and to host buffers.

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
    ap.add_argument("--costmodel-eval", action="store_true",
                    help="run the learned-fusion evaluation (4000 timings at 28 qubits, circuits of 28-34 qubits) "
                         "instead of the benchmark")
    ap.add_argument("--adjoint-fd", default="subset", choices=["subset", "all"],
                    help="FP64 central differences on a seeded 64-parameter subset, or (all) on all 624 "
                         "parameters, running the adjoint configuration alone")
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


def load_workloads():
    """The package's workload generators without the engine library: a stand-in package
    object whose __init__ (which loads libqi_gb300.so) is never run, so the reference arm
    maps no engine code."""
    import importlib
    import types
    name = "_qi_workloads_only"
    if name not in sys.modules:
        pkg = types.ModuleType(name)
        pkg.__path__ = [os.path.join(ROOT, "quant-iron_gb300")]
        sys.modules[name] = pkg
    return importlib.import_module(name + ".workloads")


GATE_CLASSES = ("1q diagonal", "1q pair", "CNOT", "controlled phase", "SWAP", "other")


def gate_class(g, kinds):
    k = int(g["kind"])
    nc = int(g["n_controls"])
    if k == kinds["SWAP"]:
        return "SWAP"
    if k == kinds["CNOT"]:
        return "CNOT"
    if k in (kinds["Z"], kinds["S"], kinds["T"], kinds["SDAG"], kinds["TDAG"], kinds["P"], kinds["RZ"],
             kinds["IDENTITY"]):
        return "controlled phase" if nc else "1q diagonal"
    if k in (kinds["H"], kinds["X"], kinds["Y"], kinds["RX"], kinds["RY"], kinds["U2"]) and nc == 0:
        return "1q pair"
    return "other"


def reference_cpu_sample(n, gates, kinds, warm, samples, threads):
    """The oracle port of the reference's rayon data flow (clone + per-pair update list +
    serial scatter, on `threads` host threads) timed gate by gate on a stratified sample of
    the circuit: sample k is a gate of class k mod 5 (1q diagonal, 1q pair, CNOT,
    controlled phase, SWAP), taken at a seeded position among that class's gates; the
    `warm` untimed gates come first.  The whole circuit's time is estimated as
    sum over classes of (gates in the class x mean sampled time of the class).
    Returns (estimated seconds per circuit, per-sample seconds, description)."""
    import numpy as np
    from oracle import oracle as orc
    by_class = {}
    for i in range(gates.size):
        by_class.setdefault(gate_class(gates[i], kinds), []).append(i)
    order = [c for c in GATE_CLASSES if c in by_class]
    rng = np.random.default_rng(12345)
    picks = []
    for k in range(warm + samples):
        c = order[k % len(order)]
        picks.append((c, by_class[c][int(rng.integers(0, len(by_class[c])))]))
    init = np.full(1 << n, 1.0 / np.sqrt(1 << n), dtype=np.complex128)
    _, secs = orc.port_execute_timed(init, n, gates[[i for _, i in picks]], threads)
    del init
    timed = list(zip([c for c, _ in picks[warm:]], secs[warm:]))
    mean_all = float(np.mean([t for _, t in timed])) if timed else 0.0
    per_class = {}
    for c in order:
        ts = [t for cc, t in timed if cc == c]
        per_class[c] = {"gates": len(by_class[c]), "sampled": len(ts),
                        "mean_s": float(np.mean(ts)) if ts else mean_all}
    est = sum(v["gates"] * v["mean_s"] for v in per_class.values())
    desc = ("oracle port of the reference rayon data flow (clone + per-pair update list + serial scatter) on %d "
            "host threads, %d qubits: %d gates timed one by one (stratified over the gate classes, %d warm-up "
            "gates untimed); circuit time = sum over classes of count x mean sampled time, extrapolation "
            "factor %.1f (%d gates / %d timed)" % (threads, n, len(timed), warm, gates.size / max(1, len(timed)),
                                                     gates.size, len(timed)))
    return est, [float(t) for _, t in timed], per_class, desc


def workload_config(n, gates, world):
    """The `config` both arms print (the same workload, whatever implements it)."""
    return {"workload": "random circuit, %d qubits, %d layers + QFT (%d gates), |+>^%d, seed %d" %
                        (n, LAYERS, gates.size, n, SEED),
            "qubits": n, "layers": LAYERS, "gates": int(gates.size),
            "l2": "inputs (%.3g GiB FP32 state) larger than the 129 MB L2; no flush" % ((1 << n) * 8 / 2**30),
            "parallelism": "replicas" if world > 1 else "single GPU"}


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


def cpu_baseline(n, gates, kinds):
    """Bounded sample (one gate per class, about 20 s at 30 qubits) of the reference CPU data flow."""
    threads = os.cpu_count() or 1
    nn = n
    while nn > 20 and host_mem_gb() < (1 << nn) * 60 / 1e9 * 1.3:   # the rayon data flow holds ~56 B/amp
        nn -= 1
    g = gates if nn == n else load_workloads().random_circuit(nn, LAYERS, seed=SEED)
    est, _, per_class, desc = reference_cpu_sample(nn, g, kinds, 0, 5, threads)
    est *= float(1 << (n - nn))   # a smaller sample scaled to n qubits by amplitude count
    if nn != n:
        desc += "; scaled by 2^%d amplitudes to %d qubits" % (n - nn, n)
    return {"value": LAYERS / est, "unit": "layers/s", "cores": threads, "kind": "port", "sample": desc,
            "seconds_per_circuit": est, "classes": per_class}


def fd_energies(qi, n, gates, theta, terms, ids, shifts, stream):
    """E(theta + s e_j) for every parameter j in ids and shift s, with the plain FP64 per-gate
    path: the state after each 77-gate layer of the unshifted circuit is kept (FP64), so an
    evaluation runs from the checkpoint before the shifted gate's layer to the end.
    Returns {(j, s): E}."""
    import numpy as np
    layer_len = 3 * n - 1
    n_layers = gates.size // layer_len
    ck = []
    st = qi.DeviceState(n, qi.F64)
    st.set_stream(stream.cuda_stream)
    st.set_zero()
    for layer in range(n_layers):
        c = qi.DeviceState(n, qi.F64)
        c.set_stream(stream.cuda_stream)
        c.copy_from(st)
        ck.append(c)
        qi.Plan(n, qi.F64, gates[layer * layer_len:(layer + 1) * layer_len], theta=theta,
                fusion=qi.FUSION_NONE).execute(st)
    pid_layer = {}
    for pos in range(gates.size):
        for k in range(3):
            pid = int(gates[pos]["param_ids"][k])
            if pid >= 0:
                pid_layer[pid] = pos // layer_len
    out = {}
    for j in ids:
        layer = pid_layer[int(j)]
        tail = gates[layer * layer_len:]
        for sgn in shifts:
            th = theta.copy()
            th[j] += sgn
            st.copy_from(ck[layer])
            qi.Plan(n, qi.F64, tail, theta=th, fusion=qi.FUSION_NONE).execute(st)
            out[(int(j), sgn)] = qi.sumop_expectation(st, terms).real
    for c in ck:
        c.close()
    st.close()
    return out


def adjoint_leg(qi, workloads, stream, torch, np, n=26, layers=12, fd="subset"):
    """Adjoint gradient of the 26-qubit hardware-efficient ansatz (12 layers of RY.RZ + CNOT
    ladder, 624 parameters, seed 1) on the periodic XXZ energy (104 terms): gradients/s with an
    FP32 state; the FP32 and FP64 adjoints on all 624 parameters; FP64 central differences
    (eps 1e-4) on a seeded 64-parameter subset (fd="all": on every parameter) and parameter shift
    (+-pi/2) on a seeded 32-parameter subset, both from the plain FP64 per-gate path."""
    gates, theta = workloads.hea_ansatz(n, layers, seed=1)
    terms = workloads.xxz_periodic(n, seed=1)
    s32 = qi.DeviceState(n, qi.F32)
    s32.set_stream(stream.cuda_stream)
    s32.set_zero()
    qi.adjoint_gradient(s32, gates, theta, terms)   # warm-up
    reps = 5
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
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e64, g64 = qi.adjoint_gradient(s64, gates, theta, terms)
    t64 = time.perf_counter() - t0
    s64.close()
    rng = np.random.default_rng(1)
    fd_ids = np.sort(rng.choice(theta.size, 64, replace=False))
    ps_ids = np.sort(rng.choice(theta.size, 32, replace=False))
    if fd == "all":
        fd_ids = np.arange(theta.size)
    t0 = time.perf_counter()
    ev = fd_energies(qi, n, gates, theta, terms, fd_ids, (1e-4, -1e-4), stream)
    ev.update(fd_energies(qi, n, gates, theta, terms, ps_ids, (np.pi / 2, -np.pi / 2), stream))
    t_ref = time.perf_counter() - t0
    g_fd = np.array([(ev[(int(j), 1e-4)] - ev[(int(j), -1e-4)]) / 2e-4 for j in fd_ids])
    g_ps = np.array([(ev[(int(j), np.pi / 2)] - ev[(int(j), -np.pi / 2)]) / 2 for j in ps_ids])

    def rel(a, b):
        return float(np.linalg.norm(a - b) / np.linalg.norm(b))
    comp = np.abs(g32[fd_ids] - g_fd) / np.maximum(np.abs(g_fd), 1e-300)
    return {"workload": "HEA %d qubits, %d layers, %d parameters, periodic XXZ (%d terms), |0>" %
                        (n, layers, theta.size, len(terms)),
            "grad_per_s_fp32": 1.0 / t_adj, "seconds_per_grad_fp32": t_adj, "seconds_per_grad_fp64": t64,
            "energy_fp32": e32, "energy_fp64": e64, "energy_error_fp32": abs(e32 - e64),
            "rel_err_fp32_vs_fp64_adjoint_all": rel(g32, g64),
            "fd": {"eps": 1e-4, "parameters": int(fd_ids.size), "source": "plain FP64 per-gate path, per-layer "
                                                                           "FP64 checkpoints",
                   "rel_err_fp32_adjoint": rel(g32[fd_ids], g_fd), "rel_err_fp64_adjoint": rel(g64[fd_ids], g_fd),
                   "max_componentwise_rel_err_fp32": float(np.max(comp)),
                   "median_componentwise_rel_err_fp32": float(np.median(comp))},
            "parameter_shift": {"parameters": int(ps_ids.size), "rel_err_fp32_adjoint": rel(g32[ps_ids], g_ps),
                                "rel_err_fp64_adjoint": rel(g64[ps_ids], g_ps)},
            "reference_seconds": t_ref,
            "norm_grad_fp64": float(np.linalg.norm(g64))}


def trotter_leg(qi, workloads, stream, torch, np, rows=5, cols=6, steps=100, observe_every=10):
    """First-order Trotter evolution on the 5x6 open lattice (30 qubits), dt = 0.05, from a
    seeded basis state, for the anisotropic Heisenberg SumOp (1.0 XX + 0.8 YY + 0.5 ZZ per bond,
    h_i Z_i; 177 terms) and the transverse-field Ising SumOp (-J_ij ZZ - g X_i, J ~ U(0.5, 1.5),
    g = 1; 79 terms).  `steps` steps of the FP32 fused method (one plan per step) and of the
    FP64 grouped method (one pass per run of terms with X-masks in {0, X}), <H> in FP64
    every `observe_every` steps for both; the energy-error trajectory FP32 - FP64."""
    n = rows * cols
    basis = int(np.random.default_rng(0).integers(0, 1 << n))
    out = {"lattice": "%dx%d open, site r*%d + c" % (rows, cols, cols), "dt": 0.05, "steps": steps,
           "observe_every": observe_every, "basis_state": basis}
    for name, terms in (("heisenberg", workloads.lattice_xyz(rows, cols, seed=0)),
                        ("tfim", workloads.lattice_tfim(rows, cols, seed=0))):
        res = {"terms": len(terms)}
        for label, prec in (("fp32_fused", qi.F32), ("fp64_grouped", qi.F64)):
            st = qi.DeviceState(n, prec)
            st.set_stream(stream.cuda_stream)
            st.set_basis(basis)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            e = qi.trotter_evolve(st, terms, 0.05, steps, observable=terms, observe_every=observe_every)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            st.close()
            res[label] = {"ms_per_step": dt * 1e3 / steps, "energies": [complex(x).real for x in e]}
        e32 = np.array(res["fp32_fused"]["energies"])
        e64 = np.array(res["fp64_grouped"]["energies"])
        res["energy_error"] = [float(x) for x in np.abs(e32 - e64)]
        res["max_energy_error"] = float(np.max(np.abs(e32 - e64)))
        res["speedup_fp32_fused_vs_fp64_grouped"] = (res["fp64_grouped"]["ms_per_step"] /
                                                     res["fp32_fused"]["ms_per_step"])
        out[name] = res
    out["note"] = "timed regions include the <H> evaluations"
    return out


def seeds_leg(qi, workloads, stream, torch, n, seeds, terms):
    """The benchmark circuit family at n qubits for several seeds: the fused complex-FP32 plan
    against the plain FP64 per-gate plan on the device — infidelity, full-state max amplitude
    error (every one of the 2^n amplitudes) and energy error (<H> of the open-chain
    Heisenberg, FP64 reductions) — with both methods' times."""
    out = []
    s64 = qi.DeviceState(n, qi.F64)
    s64.set_stream(stream.cuda_stream)
    s32 = qi.DeviceState(n, qi.F32)
    s32.set_stream(stream.cuda_stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for seed in seeds:
        gates = workloads.random_circuit(n, LAYERS, seed=seed)
        p64 = qi.Plan(n, qi.F64, gates, fusion=qi.FUSION_NONE)
        p32 = qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=FUSED_K)
        s64.set_plus()
        torch.cuda.synchronize()
        e0.record(stream)
        p64.execute(s64)
        e1.record(stream)
        torch.cuda.synchronize()
        ms64 = e0.elapsed_time(e1)
        s32.set_plus()
        torch.cuda.synchronize()
        e0.record(stream)
        p32.execute(s32)
        e1.record(stream)
        torch.cuda.synchronize()
        ms32 = e0.elapsed_time(e1)
        cmp = s32.compare(s64)
        en32 = qi.sumop_expectation(s32, terms).real
        en64 = qi.sumop_expectation(s64, terms).real
        out.append({"seed": seed, "fused_fp32_ms": ms32, "fp64_per_gate_ms": ms64, "speedup": ms64 / ms32,
                    "infidelity": cmp["infidelity"], "max_amp_error": cmp["max_abs_err"],
                    "energy_fp32": en32, "energy_fp64": en64, "energy_error": abs(en32 - en64),
                    "plan_kernels": p32.stats()["n_kernels"]})
        del p64, p32
    s64.close()
    s32.close()
    return out


def per_gate_leg(qi, workloads, stream, n, peak):
    """One kernel per gate at n qubits (the plain method's kernels) by gate kind and target
    qubit, FP32 and FP64: CUDA-event time per launch (qi_plan_profile), achieved bandwidth on
    the full-pass convention (16 / 32 B per amplitude) and on the bytes the kernel must move
    (diagonal gates and CNOTs touch half of the amplitudes, a controlled phase a quarter)."""
    gl = workloads.GateList()
    cases = []
    for q in (0, 1, 3, 5, 8, 16, n - 1):
        gl.add("H", [q]); cases.append(("H (pair)", q, 1.0))
        gl.add("RY", [q], [], [0.3]); cases.append(("RY (real pair)", q, 1.0))
        gl.add("RX", [q], [], [0.3]); cases.append(("RX (general pair)", q, 1.0))
        gl.add("RZ", [q], [], [0.3]); cases.append(("RZ (diagonal)", q, 1.0))
        gl.add("T", [q]); cases.append(("T (phase on |1>)", q, 0.5))
    for q in (0, 4, 16, n - 2):
        gl.add("CNOT", [q + 1], [q]); cases.append(("CNOT", q, 0.5))
        gl.add("P", [q + 1], [q], [0.3]); cases.append(("controlled phase", q, 0.25))
        gl.add("SWAP", [q, q + 1]); cases.append(("SWAP", q, 0.5))
    gates = gl.array()
    out = {}
    for label, prec, amp in (("fp32", qi.F32, 8), ("fp64", qi.F64, 16)):
        plan = qi.Plan(n, prec, gates, fusion=qi.FUSION_NONE)
        st = qi.DeviceState(n, prec)
        st.set_stream(stream.cuda_stream)
        st.set_plus()
        qi.plan_profile(plan, st)   # warm-up
        ops, ms = qi.plan_profile(plan, st)
        rows = []
        for (kind, q, frac), t in zip(cases, ms):
            full = (1 << n) * amp * 2
            rows.append({"gate": kind, "qubit": q, "ms": t, "full_pass_gbs": full / (t / 1e3) / 1e9,
                         "full_pass_frac": full / (t / 1e3) / 1e9 / peak,
                         "touched_gbs": frac * full / (t / 1e3) / 1e9,
                         "touched_frac": frac * full / (t / 1e3) / 1e9 / peak})
        out[label] = rows
        st.close()
    return out


def costmodel_eval(qi, workloads, torch, np, n_train=28, count=4000, qubits=range(28, 35), exhaustive_upto=30,
                   per_size=3):
    """The learned-fusion configuration: the cost model trained on `count` engine-timed blocks
    at n_train qubits, then seeded random circuits of the benchmark family (`per_size` per qubit
    count in `qubits`, depth 20-60) planned three ways — greedy fixed-k, the learned choice, and (up to
    `exhaustive_upto` qubits) exhaustive timing of every preset partition — compared by measured
    wall time, and the learned plan's infidelity against the FP64 per-gate path up to
    33 qubits (FP64 at 34 qubits would need 256 GiB); the exhaustive timing and the FP64 check run
    on the first circuit of each qubit count."""
    from quant_iron_gb300 import costmodel
    t0 = time.perf_counter()
    X, y = costmodel.collect(n_train, count, seed=11)
    t_collect = time.perf_counter() - t0
    idx = np.random.default_rng(0).permutation(len(y))
    cut = int(0.9 * len(y))
    hist = costmodel.train(X[idx[:cut]], y[idx[:cut]], epochs=2000, lr=3e-3, seed=1)
    pred = costmodel.predict(X[idx[cut:]])
    out = {"training": {"qubits": n_train, "timings": int(count), "collect_s": t_collect,
                        "loss_first": float(hist[0]), "loss_last": float(hist[-1]),
                        "holdout_corr": float(np.corrcoef(pred, y[idx[cut:]])[0, 1]),
                        "holdout_rmse_log_ms": float(np.sqrt(np.mean((pred - y[idx[cut:]]) ** 2)))},
           "circuits": []}

    def timed(plan, st, reps=2):
        st.set_plus()
        plan.execute(st)
        st.synchronize()
        best = 1e30
        for _ in range(reps):
            st.set_plus()
            st.synchronize()
            t1 = time.perf_counter()
            plan.execute(st)
            st.synchronize()
            best = min(best, time.perf_counter() - t1)
        return best * 1e3

    for n, rep in ((n, rep) for n in qubits for rep in range(per_size)):
        depth = 20 + (7 * n + 13 * rep) % 41
        gates = workloads.random_circuit(n, depth, seed=100 + n + 1000 * rep)
        st = qi.DeviceState(n, qi.F32)
        rec = {"qubits": n, "layers": depth, "gates": int(gates.size), "seed": 100 + n + 1000 * rep}
        pg = qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=6)
        rec["greedy_ms"] = timed(pg, st)
        t1 = time.perf_counter()
        pl = qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_LEARNED, max_block_qubits=6)
        rec["learned_plan_build_s"] = time.perf_counter() - t1
        rec["learned_ms"] = timed(pl, st)
        rec["learned_predicted_ms"] = pl.stats()["predicted_us"] / 1e3
        rec["learned_kernels"] = pl.stats()["n_kernels"]
        rec["greedy_kernels"] = pg.stats()["n_kernels"]
        if n <= exhaustive_upto and rep == 0:
            ex = {}
            for k in (2, 3, 4, 5, 6):
                for tc in ((0, 2) if k >= 5 else (2,)):
                    ex["k%d%s" % (k, "_tc" if tc == 0 else "")] = timed(
                        qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=k, use_tensor_cores=tc), st)
            ex["per_gate"] = timed(qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_NONE), st, reps=1)
            rec["exhaustive_ms"] = ex
            rec["exhaustive_best"] = min(ex, key=ex.get)
            rec["exhaustive_best_ms"] = ex[rec["exhaustive_best"]]
        if n <= 33 and rep == 0:
            s64 = qi.DeviceState(n, qi.F64)
            s64.set_plus()
            qi.Plan(n, qi.F64, gates, fusion=qi.FUSION_NONE).execute(s64)
            st.set_plus()
            pl.execute(st)
            rec["learned_infidelity"] = st.compare(s64)["infidelity"]
            s64.close()
        st.close()
        out["circuits"].append(rec)
        print(json.dumps(rec), file=sys.stderr, flush=True)
    c = out["circuits"]
    ratios = [x["learned_ms"] / x["greedy_ms"] for x in c]
    out["summary"] = {"circuits": len(c), "learned_over_greedy_wall": ratios,
                      "geomean_learned_over_greedy": float(np.exp(np.mean(np.log(ratios)))),
                      "worst_learned_over_greedy": max(ratios),
                      "learned_over_exhaustive_best": [x["learned_ms"] / x["exhaustive_best_ms"] for x in c
                                                       if "exhaustive_best_ms" in x],
                      "max_infidelity": max(x.get("learned_infidelity", 0.0) for x in c)}
    return out


def run_reference(args):
    """The reference implementation's CPU path (the oracle port of its rayon data flow; the
    crate itself needs a Rust toolchain, absent on both machines) on this workload.  A step
    is one gate of the circuit, timed on its own, cycling over the gate classes; `value`
    is the whole circuit's layers/s estimated from the per-class mean times, and
    ms_per_step is the mean time of the timed gates.  No engine code is loaded."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import __graft_entry__ as ge
    ge.build_oracle()
    workloads = load_workloads()
    from _qi_workloads_only._types import GATE_KINDS
    n = args.qubits
    gates = workloads.random_circuit(n, LAYERS, seed=SEED)
    threads = os.cpu_count() or 1
    nn = n
    while nn > 20 and host_mem_gb() < (1 << nn) * 60 / 1e9 * 1.3:
        nn -= 1
    g = gates if nn == n else workloads.random_circuit(nn, LAYERS, seed=SEED)
    est, secs, per_class, desc = reference_cpu_sample(nn, g, GATE_KINDS, args.warmup, args.steps, threads)
    est *= float(1 << (n - nn))
    if nn != n:
        desc += "; scaled by 2^%d amplitudes to %d qubits" % (n - nn, n)
    value = LAYERS / est
    world = int(os.environ.get("WORLD_SIZE", "1"))
    line = {"impl": "reference", "metric": "layers/s", "value": value, "unit": "layers/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(secs) / max(1, len(secs)),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "c128", "data": "synthetic",
            "config": workload_config(n, gates, world),
            "step": "one gate of the circuit on the reference CPU data flow (stratified over gate classes)",
            "estimated_seconds_per_circuit": est, "classes": per_class,
            "cpu_baseline": {"value": value, "unit": "layers/s", "cores": threads, "kind": "port", "sample": desc},
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

    if args.costmodel_eval:
        print(json.dumps(costmodel_eval(qi, workloads, torch, np)))
        return
    if args.adjoint_fd == "all":   # the adjoint configuration alone, every parameter checked
        print(json.dumps(adjoint_leg(qi, workloads, torch.cuda.Stream(), torch, np, fd="all")))
        return
    n = args.qubits
    gates = workloads.random_circuit(n, LAYERS, seed=SEED)
    terms = workloads.heisenberg_open_chain(n, seed=SEED)
    t0 = time.perf_counter()
    plan = qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_GREEDY, max_block_qubits=FUSED_K)
    plan_s = time.perf_counter() - t0
    stats = plan.stats()
    # high priority: in the e2e pipeline the uploads the GPU reads over the link run on the engine's
    # lowest-priority stream, so the circuits get freed SMs first
    stream = torch.cuda.Stream(priority=-1)
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
        traffic_src = "ncu dram__bytes_read.sum + dram__bytes_write.sum of a 26-qubit k_fused_tc launch, x 2^%d" % (n - 26)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "traffic_source": traffic_src, "kernel": dom, "peak_source": peak_kind,
                "algorithmic_bytes_per_launch": pass_bytes, "avg_launch_ms": avg_ms,
                "kernels": {k: {"launches": v["launches"], "ms": round(v["ms"], 3),
                                "share": round(v["ms"] / max(1e-9, sum(x["ms"] for x in by_kernel.values())), 4)}
                            for k, v in by_kernel.items()}}
    if dom == "k_fused_tc":
        # the same kernel against the tensor roof: 3 split products x 8 * 2^k flop per amplitude
        # (k = 6: 1536 flop/amp) per launch; peak = the dense tcgen05 kind::tf32 rate measured
        # here by the engine's own probe kernel (MEASURED_PEAKS.json holds no TF32 figure)
        probe_clk = ClockSampler(local)
        probe_clk.start()
        tf32_peak, probe_ms = qi.tf32_rate_probe(iters=65536, reps=40)   # ~0.2 s: clocks sampled under load
        pclk = probe_clk.stop()
        tflop = 3 * 8 * (1 << FUSED_K) * (1 << n) / 1e12
        roofline["tensor"] = {"achieved": tflop / (avg_ms / 1e3), "peak": tf32_peak, "unit": "TFLOP/s",
                              "frac": tflop / (avg_ms / 1e3) / tf32_peak,
                              "peak_source": "measured here: qi_tf32_rate_probe (tcgen05.mma kind::tf32 M128 N256 "
                                             "K8, one CTA per SM, best of 40 launches of %.2f ms)" % probe_ms,
                              "peak_clocks": pclk, "flop_per_amp": 3 * 8 * (1 << FUSED_K)}

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
        # the benchmark family on 5 seeds: fused FP32 against the plain FP64 per-gate path
        # (the >= 8x target's denominator), full-state errors; seed 0 is the headline circuit
        seeds = seeds_leg(qi, workloads, stream, torch, n, list(range(5)), terms)
        s0 = seeds[0]
        plan32 = qi.Plan(n, qi.F32, gates, fusion=qi.FUSION_NONE)
        st.set_plus()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plan32.execute(st)
        e1.record(stream)
        torch.cuda.synchronize()
        ms32 = e0.elapsed_time(e1)
        del plan32
        extra = {"fp64_per_gate_ms": s0["fp64_per_gate_ms"], "fp32_per_gate_ms": ms32, "fused_fp32_ms": ms_per_step,
                 "speedup_fused_vs_fp64_per_gate": s0["fp64_per_gate_ms"] / ms_per_step,
                 "infidelity_fused_vs_fp64": s0["infidelity"], "max_amp_error_full_state": s0["max_amp_error"],
                 "energy_fused_fp32": s0["energy_fp32"], "energy_fp64_per_gate": s0["energy_fp64"],
                 "energy_error": s0["energy_error"], "gates_per_s_fused": len(gates) / (ms_per_step / 1e3),
                 "seeds": seeds,
                 "worst_over_seeds": {"infidelity": max(x["infidelity"] for x in seeds),
                                      "max_amp_error": max(x["max_amp_error"] for x in seeds),
                                      "energy_error": max(x["energy_error"] for x in seeds),
                                      "speedup": min(x["speedup"] for x in seeds)}}
        extra["per_gate"] = per_gate_leg(qi, workloads, stream, n, peak)
        extra["adjoint"] = adjoint_leg(qi, workloads, stream, torch, np)
        extra["trotter"] = trotter_leg(qi, workloads, stream, torch, np)
    extra["expectation"] = expectation

    # end-to-end through the public API with host buffers: H2D of the initial state,
    # the circuit, D2H of the final state, every step.  Two device states alternate: each
    # step's download runs on the copy engine (page-locked buffers) while the other state's
    # circuit runs; the upload takes one of the two public paths, chosen by a short trial of
    # each on this machine's link (below).
    e2e = None
    if rank == 0:
        dim = 1 << n
        pipelined = host_mem_gb() > 3.5 * 16 * dim / 1e9
        host_in = torch.empty(2 * dim, dtype=torch.float64, pin_memory=True)
        host_in.fill_(1.0 / (dim ** 0.5))
        host_in[1::2] = 0.0
        if pipelined:
            host_out = [torch.empty(2 * dim, dtype=torch.float64, pin_memory=True) for _ in range(2)]
            stream2 = torch.cuda.Stream(priority=-1)
            st2 = qi.DeviceState(n, qi.F32)
            st2.set_stream(stream2.cuda_stream)
            states = [st, st2]
            for s2 in states:   # allocates each state's staging and second buffers (an allocation synchronises
                s2.upload_async(host_in.data_ptr(), dim)   # the device, so none may happen in the timed loop)
                plan.execute(s2)
                s2.synchronize()
            # the host link on its own: the copy engine both ways, and the GPU reading the page-locked
            # buffer itself over the link (qi_state_upload; converts as it reads, uses the SMs)
            link = {}
            for name, fn in (("h2d_ms", lambda: st.upload_async(host_in.data_ptr(), dim)),
                             ("d2h_ms", lambda: st.download_async(host_out[0].data_ptr(), dim)),
                             ("h2d_sm_ms", lambda: st.upload_ptr(host_in.data_ptr(), dim)),
                             ("d2h_sm_ms", lambda: st.download_ptr(host_out[0].data_ptr(), dim))):
                torch.cuda.synchronize()
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(stream)
                fn()
                b.record(stream)
                torch.cuda.synchronize()
                link[name] = a.elapsed_time(b)
            for k in ("h2d", "d2h", "h2d_sm", "d2h_sm"):
                link[k + "_gbs"] = 16 * dim / (link[k + "_ms"] / 1e3) / 1e9

        def run_pipeline(sm_link, steps):
            """`steps` circuits one after the other (each state waits for the other's circuit, not
            for its download), each state's download and next upload overlapping the other state's
            circuit; downloads on the copy engine, uploads on the copy engine too or, with
            `sm_link`, read by the GPU over the link (upload_ptr; downloads made that way competed
            with the other state's circuit: 357 against 311 ms per step on a 185 GB/s box).
            Returns (device ms from the first upload to the last download, circuit end ms)."""
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            circuit_end = []
            for k in range(steps):
                s2, other = states[k % 2], states[(k + 1) % 2]
                if sm_link:
                    s2.upload_ptr(host_in.data_ptr(), dim)
                else:
                    s2.upload_async(host_in.data_ptr(), dim)
                if k > 0:
                    s2.wait_for(other)   # other's stream so far ends with its circuit
                plan.execute(s2)
                ce = torch.cuda.Event(enable_timing=True)
                ce.record(stream if k % 2 == 0 else stream2)
                circuit_end.append(ce)
                if k > 0:
                    other.download_async(host_out[(k - 1) % 2].data_ptr(), dim)
            states[(steps - 1) % 2].download_async(host_out[(steps - 1) % 2].data_ptr(), dim)
            joined = torch.cuda.Event()
            joined.record(stream2)
            stream.wait_event(joined)
            e1.record(stream)
            torch.cuda.synchronize()
            return e0.elapsed_time(e1), [e0.elapsed_time(c) for c in circuit_end]

        sm_link = False
        if pipelined:
            trial = {}
            for mode in (False, True):
                ms, _ = run_pipeline(mode, 3)
                trial["gpu_reads_upload" if mode else "copy_engines"] = ms / 3
            sm_link = trial["gpu_reads_upload"] < trial["copy_engines"]
            link["trial_ms_per_step"] = trial
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if pipelined:
            # ten circuits at least, so that the pipeline's fill (the first upload) and drain
            # (the last download) weigh less than in a five-step run
            e2e_steps = max(10, args.steps)
            e2e_ms, ends = run_pipeline(sm_link, e2e_steps)
        else:   # not enough page-locked host memory for two output buffers: one state, in order
            e2e_steps = max(1, min(args.steps, 3))
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(e2e_steps):
                st.upload_ptr(host_in.data_ptr(), dim)
                plan.execute(st)
                st.download_ptr(host_in.data_ptr(), dim)
            e1.record(stream)
            torch.cuda.synchronize()
            e2e_ms = e0.elapsed_time(e1)
        wall = time.perf_counter() - t0
        e2e = {"value": LAYERS * e2e_steps / (e2e_ms / 1e3), "unit": "layers/s", "h2d_bytes_per_step": 16 * dim,
               "d2h_bytes_per_step": 16 * dim, "wall_s": wall, "steps": e2e_steps,
               "pipeline": (("two device states, circuits in turn (qi_state_wait); " +
                             ("uploads read by the GPU over the link (qi_state_upload, lowest-priority stream), "
                              "downloads on the copy engine, beside the other state's circuit"
                              if sm_link else
                              "each state's H2D and D2H on the copy engines overlap the other state's circuit") +
                             "; transfer path chosen by a 3-step trial of each")
                            if pipelined else "one state, transfers in order")}
        if pipelined:
            e2e["link"] = link
            e2e["circuit_end_ms"] = [round(x, 1) for x in ends]
            e2e["steady_ms_per_step"] = (ends[-1] - ends[0]) / max(1, len(ends) - 1)
            st2.close()
            del host_out
        del host_in

    cpu = None
    if rank == 0 and world == 1 and not args.skip_baselines:
        st.close()
        cpu = cpu_baseline(n, gates, qi._abi.GATE_KINDS)

    if rank == 0:
        line = {"metric": "layers/s", "value": value, "unit": "layers/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "c64", "data": "synthetic",
                "config": workload_config(n, gates, world),
                "method": {"precision": "complex FP32 state, FP64 reductions", "fusion": "greedy k<=%d" % FUSED_K,
                           "tensor_cores": "3xTF32 tcgen05 for blocks of k >= 5", "plan": stats,
                           "plan_build_s": plan_s},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clk, "gpu_launches": launches}
        line.update(extra)
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()

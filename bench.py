"""GAP-SOAP energy+force+virial throughput on one GB300 (atom-evals/s).

One "step" is one full evaluation (neighbour list, SOAP and gradients, sparse-GP
kernel GEMMs, forces, virial) of one structure of the chosen workload:
  si4096   4096-atom Si diamond 8x8x8 (a=5.43 A, rattle N(0, 0.1 A)); SOAP n_max=8
           l_max=6 rc=5 A (D=253), 2000 sparse points, zeta=4, + distance_2b (20 points).
  sic32768 32768-atom random Si/C cell (50/50, 3.2 g/cm^3, 1.6 A minimum separation);
           SOAP n_max=10 l_max=8 rc=5 A with 2 species channels (D=1891), 8000 sparse
           points, zeta=4, + distance_2b per species pair.
  sic8192  the same model on an 8192-atom cell (the size used for ncu captures).
The headline runs in the precision given (default fp16: FP32 SOAP, both sparse-GP GEMMs
with FP16 operands on tcgen05); the same line carries, on the same structure,
  fp64     the plain FP64 path: throughput and every mixed form's error against it;
  forms    the other mixed forms (tf32: both GEMMs in TF32; bf16x3: split-BF16, three
           products): throughput, stage times and errors, each against its own ceiling;
  cpu_baseline  the FP64 CPU restatement (oracle/) on the host cores, on a sample of
           centres, and every form's error against it on those centres;
and, each in a child process with its own wall-clock budget (killed when it runs out,
reported as skipped), so that the line is always printed:
  batch    1024 independent triclinic Si/C structures (atom counts log-uniform in
           [8, 2048], lengths 4-30 A, angles 70-110 deg, 1.8 A minimum separation) in one
           batched evaluation, first call and CUDA-graph replay, against the plain FP64
           per-structure loop on a sample;
  serving  Poisson streams of E+F requests (sizes log-uniform 16-2048, drawn as for
           batch) at several offered loads, served by the continuous-batching server
           while 64 resident 512-atom Si MD replicas (1000 K, dt = 1 fs, 0.5 A skin)
           step on their own stream; p50/p99 latency and throughput per load.
Inputs are seeded synthetic structures and random GAP models (no dataset is published
for this path).  `value` is timed with CUDA events on the launching stream with the
inputs resident in HBM; `e2e` goes through the public C ABI (gapgpu_calc) with pinned
host buffers, host<->device copies inside the timed region.  L2 is flushed (256 MB
write) between timed steps.  `--impl reference` times the FP64 CPU restatement of the
reference (oracle/) on the host cores.  Progress goes to stderr with elapsed times.
"""
import argparse
import contextlib
import json
import os
import signal
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "GAP-SOAP atom-evals/s E+F, mixed vs FP64 on GB300 at <=1 meV/A; p50/p99 latency"
STAGES = ["neighbours", "soap_fwd", "gemm", "soap_bwd", "pair2b", "reduce", "total"]
T_START = time.perf_counter()


def log(msg):
    sys.stderr.write("[bench %7.1fs] %s\n" % (time.perf_counter() - T_START, msg))
    sys.stderr.flush()


def peaks():
    try:
        return json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "fallback": True}


WORKLOADS = {
    "si4096": dict(kind="si", n_rep=8, rattle=0.1, n_max=8, l_max=6, cutoff=5.0, M=2000, species=(14,), seed=11),
    "si64": dict(kind="si", n_rep=2, rattle=0.05, n_max=8, l_max=6, cutoff=5.0, M=500, species=(14,), seed=7),
    "sic32768": dict(kind="sic", n=32768, n_max=10, l_max=8, cutoff=5.0, M=8000, species=(14, 6), seed=21),
    # the sic32768 model on an 8192-atom cell: the profiling case (per-kernel inputs still above L2)
    "sic8192": dict(kind="sic", n=8192, n_max=10, l_max=8, cutoff=5.0, M=8000, species=(14, 6), seed=21),
}

# what each precision runs: the arithmetic named in the line's config and dtype
PRECISION_TEXT = {
    "fp64": "plain FP64 (SOAP, GEMMs, reductions)",
    "fp16": "FP32 SOAP; both sparse-GP GEMMs with FP16 operands (10-bit mantissas) on tcgen05, FP32 accumulation",
    "tf32": "FP32 SOAP; both sparse-GP GEMMs in TF32 on tcgen05, FP32 accumulation",
    "bf16x3": "FP32 SOAP; both sparse-GP GEMMs in split-BF16 (hi*hi + hi*lo + lo*hi) on tcgen05, FP32 accumulation",
}
DTYPE = {"fp64": "f64", "fp16": "f32+f16", "tf32": "f32+tf32", "bf16x3": "f32+bf16x3"}


def make_structure(w):
    from quip_gb300 import models
    if w["kind"] == "si":
        return models.si_diamond(w["n_rep"], rattle=w["rattle"], seed=w["seed"])
    return models.random_binary(w["n"], seed=w["seed"])


def make_model(w, tmpdir, descriptor_fn):
    from quip_gb300 import models
    if w["kind"] == "si":
        structs = [models.si_diamond(4, rattle=0.05 + 0.03 * k, seed=200 + k) for k in range(max(1, w["M"] // 512 + 1))]
    else:
        structs = [models.random_binary(2048, seed=300 + k) for k in range(w["M"] // 2048 + 1)]
    return models.random_soap_gap(os.path.join(tmpdir, "bench_gap.xml"), descriptor_fn, structs, n_max=w["n_max"],
                                  l_max=w["l_max"], cutoff=w["cutoff"], width=1.0, atom_sigma=0.5,
                                  species=w["species"], M=w["M"], zeta=4.0, delta=1.0, seed=w["seed"])


def soap_sizes(w):
    n, L = w["n_max"], w["l_max"] + 1
    N = n * len(w["species"])
    P = N * (N + 1) // 2
    return n, L, N, P, P * L + 1


def algorithmic_flops(w, nu):
    """Per-atom FLOPs of one evaluation (canonical count): expansion, power spectrum,
    kernel + weight GEMMs, adjoint to c, force contraction."""
    n, L, N, P, D = soap_sizes(w)
    M = w["M"]
    gemm = 2 * (2 * D * M)
    return 2 * (nu * n * L * L + P * L * L + N * N * L * L + 3 * nu * n * L * L) + gemm, gemm


def stage_flops(w, nu):
    """The canonical count split by stage (per centre): the forward kernel does the
    expansion and the power spectrum, the backward kernel the adjoint to c and the
    force contraction, the GEMM stage the two kernel GEMMs."""
    n, L, N, P, D = soap_sizes(w)
    return {"soap_fwd": 2 * (nu * n * L * L + P * L * L), "gemm": 4 * D * w["M"],
            "soap_bwd": 2 * (N * N * L * L + 3 * nu * n * L * L)}


class Clocks:
    def __init__(self, path):
        self.path = path
        self.p = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            self.p.wait()
            self.f.close()

    def summary(self):
        try:
            rows = [l.split(",") for l in open(self.path).read().strip().splitlines() if l.strip()]
            rows = [r for r in rows if r[0].strip() == rows[0][0].strip()]
            sm = [float(r[1]) for r in rows]
            mx = max(float(r[2]) for r in rows)
            reasons = set()
            names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
            for r in rows:
                for k, nm in enumerate(names):
                    if r[5 + k].strip() == "Active":
                        reasons.add(nm)
            return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(rows)}
        except Exception as e:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "error": str(e)[:80]}


class NvmlClocks:
    """SM clock and clock-event reasons of this process's GPU read through NVML
    (libnvidia-ml, the library nvidia-smi reads) every `period` seconds in a thread, so
    that a timed region of a few tens of milliseconds still gets several samples.  Read
    only: nothing is set."""
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown",
               0x80: "hw_power_brake_slowdown"}

    def __init__(self, period=0.01):
        import ctypes
        import torch
        self.ct, self.period = ctypes, period
        self.L = ctypes.CDLL("libnvidia-ml.so.1")
        if self.L.nvmlInit_v2() != 0:
            raise RuntimeError("nvmlInit failed")
        self.h = ctypes.c_void_p()
        props = torch.cuda.get_device_properties(torch.cuda.current_device())
        rc = self.L.nvmlDeviceGetHandleByUUID(("GPU-%s" % props.uuid).encode(), ctypes.byref(self.h))
        if rc != 0:
            bus = "%08X:%02X:%02X.0" % (props.pci_domain_id, props.pci_bus_id, props.pci_device_id)
            rc = self.L.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(), ctypes.byref(self.h))
        if rc != 0:
            raise RuntimeError("no NVML handle for this GPU (%d)" % rc)
        self.reasons_fn = getattr(self.L, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.L.nvmlDeviceGetCurrentClocksThrottleReasons
        mx = ctypes.c_uint()
        self.L.nvmlDeviceGetMaxClockInfo(self.h, 1, ctypes.byref(mx))   # NVML_CLOCK_SM
        self.max_mhz = float(mx.value)
        self.samples = []

    def _poll(self):
        ct = self.ct
        mhz, reasons = ct.c_uint(), ct.c_ulonglong()
        while not self.stop.is_set():
            if self.L.nvmlDeviceGetClockInfo(self.h, 1, ct.byref(mhz)) == 0 and \
                    self.reasons_fn(self.h, ct.byref(reasons)) == 0:
                self.samples.append((float(mhz.value), int(reasons.value)))
            self.stop.wait(self.period)

    def __enter__(self):
        import threading
        self.stop = threading.Event()
        self.t = threading.Thread(target=self._poll, daemon=True)
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop.set()
        self.t.join(timeout=5)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": self.max_mhz, "reasons": [], "samples": 0, "source": "nvml"}
        reasons = sorted({nm for _, r in self.samples for bit, nm in self.REASONS.items() if r & bit})
        return {"sm_mhz": float(np.median([m for m, _ in self.samples])), "sm_max_mhz": self.max_mhz,
                "reasons": reasons, "samples": len(self.samples),
                "source": "NVML every %g ms during the timed steps" % (1e3 * self.period)}


def clock_sampler(path):
    """NvmlClocks, else nvidia-smi every 200 ms (Clocks)."""
    try:
        return NvmlClocks()
    except Exception as e:
        log("clocks: NVML unavailable (%s), sampling with nvidia-smi" % str(e)[:80])
        return Clocks(path)


def cpu_model():
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in open("/proc/cpuinfo"):
            if line.lower().startswith(("model name", "cpu part")):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


CPU_KEYS = ("value", "unit", "cores", "kind", "sample", "seconds_fixed", "seconds_per_centre")
# centres timed at the large workloads: 1/16 of the 32768-atom cell (one oracle call over all
# 32768 centres takes about a minute on 16 cores; the per-centre cost of a 256-centre sample
# understated it by a quarter, that of a 2048-centre sample tracks it closely)
CPU_SAMPLE = 2048


def cpu_reference(w, at, model_path, steps, warmup, sample_atoms=None, nthreads=None, keep=None):
    """Times the FP64 CPU restatement (oracle) on the host cores.

    With a sample of centres, a call costs a part paid once per structure (the neighbour
    list of all N atoms and the set-up) plus a part per evaluated centre.  Both are timed:
    a call with no centres gives the first, the sampled call minus it the second, and the
    value is the full structure's rate N / (fixed + N * per-centre), so that the fixed
    part is spread over all N centres as in a full evaluation, not over the sample.
    `keep` (a dict) receives the last sampled call's results and its mask."""
    from oracle import oracle
    om = oracle.OracleModel.from_xml(model_path)
    n = len(at)
    mask = None
    ncent = n
    if sample_atoms and sample_atoms < n:
        mask = np.zeros(n, np.int32)
        mask[np.random.default_rng(0).choice(n, sample_atoms, replace=False)] = 1
        ncent = sample_atoms
    cores = nthreads or os.cpu_count()

    def timed(m, reps):
        ts = []
        for _ in range(reps):
            t0 = time.perf_counter()
            res = om.calc(at.positions, at.numbers, at.lattice, [1, 1, 1], mask=m, nthreads=cores)
            ts.append(time.perf_counter() - t0)
            if keep is not None and m is mask:
                keep["result"], keep["mask"] = res, mask
        return float(np.median(ts))

    for _ in range(warmup):
        om.calc(at.positions, at.numbers, at.lattice, [1, 1, 1], mask=mask, nthreads=cores)
    t = timed(mask, steps)
    out = {"unit": "atom-evals/s", "cores": cores, "kind": "port", "seconds_per_sample": t}
    if mask is None:
        out["value"] = n / t
        out["sample"] = "all %d centres of the %s workload, median of %d" % (n, w["name"], steps)
        return out
    t_fixed = timed(np.zeros(n, np.int32), min(steps, 3))  # its median needs few repeats
    t_centre = (t - t_fixed) / ncent
    if t_centre <= 0:  # timing noise larger than the centres' work: no extrapolation
        out["value"] = ncent / t
        out["sample"] = "%d of %d centres of the %s workload, median of %d" % (ncent, n, w["name"], steps)
        return out
    out["value"] = n / (t_fixed + n * t_centre)
    out["sample"] = ("%d of %d centres of the %s workload (median of %d: %.3f s) and the same call with no centres "
                     "(%.3f s: neighbour list and set-up); value = %d / (fixed + %d x per-centre)"
                     % (ncent, n, w["name"], steps, t, t_fixed, n, n))
    out["seconds_fixed"] = t_fixed
    out["seconds_per_centre"] = t_centre
    return out


def max_over_ranks(t_local):
    """The job's time under torchrun: the slowest rank's (replicas run independently;
    this is the only collective, outside the timed region)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(t_local)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(t_local)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------- batch and serving legs
def measure_batch(path, precision, structs, fp64_sample=48):
    """One batched evaluation of all structures (host arrays in and out, wall clock):
    first call, then repeated calls with CUDA-graph replay; the per-structure FP64 loop
    on a sample for comparison; the mixed result's error against it on that sample."""
    from quip_gb300.potential import Potential
    natoms = sum(len(a) for a in structs)
    pot = Potential(param_filename=path, precision=precision)
    t0 = time.perf_counter()
    res = pot.calc_batch(structs)
    first = time.perf_counter() - t0
    log("batch: first call %.3f s" % first)
    pot.set_option("graphs", 1)
    pot.set_option("timing", 0)
    reps = []
    for _ in range(4):   # direct, capture, replay, replay
        t0 = time.perf_counter()
        pot.calc_batch(structs)
        reps.append(time.perf_counter() - t0)
    log("batch: repeats %s" % ["%.3f" % r for r in reps])
    p64 = Potential(param_filename=path, precision="fp64")
    sample = structs[:fp64_sample]
    t0 = time.perf_counter()
    r64 = [p64.calc(a) for a in sample]
    t64 = time.perf_counter() - t0
    n64 = sum(len(a) for a in sample)
    fmax = max(float(np.abs(r["force"] - b["force"]).max()) for r, b in zip(r64, res[:fp64_sample]) if len(r["force"]))
    emax = max(abs(r["energy"] - b["energy"]) / max(1, len(a)) for r, b, a in zip(r64, res[:fp64_sample], sample))
    return {"structures": len(structs), "atoms": natoms, "precision": precision,
            "first_call_s": first, "atom_evals_per_s_first": natoms / first,
            "graph_replay_s": min(reps[2:]), "atom_evals_per_s": natoms / min(reps[2:]),
            "fp64_loop": {"structures": len(sample), "atoms": n64, "seconds": t64, "atom_evals_per_s": n64 / t64},
            "speedup_vs_fp64_loop": (natoms / min(reps[2:])) / (n64 / t64),
            "error_vs_fp64_sample": {"force_max_eV_per_A": fmax, "energy_per_atom_eV": emax},
            "timing": "wall clock around gapgpu_calc_batch with host arrays (copies included)"}


def measure_serving(path, precision, pool, loads, seconds, replicas=64, seed=11, report=None):
    """Continuous-batching serving of Poisson request streams (sizes log-uniform 16-2048,
    drawn from `pool`) next to resident MD replicas of 512-atom Si at 1000 K.  `report`
    is called with the results so far after every load."""
    from quip_gb300 import models as mdl
    from quip_gb300.md import MDReplicas
    from quip_gb300.potential import Potential
    from quip_gb300.serving import Server, poisson_arrivals
    reqpool = [a for a in pool if 16 <= len(a) <= 2048]
    md = MDReplicas(Potential(param_filename=path, precision=precision),
                    [mdl.si_diamond(4, rattle=0.05, seed=500 + k) for k in range(replicas)], dt=1.0, skin=0.5,
                    temperature=1000.0, seed=seed)
    srv = Server(path, precision=precision, workers=2, budget_bytes=24 << 30, md=md)
    t0 = time.perf_counter()
    srv.warmup(reqpool)
    warm = time.perf_counter() - t0
    log("serving: warm-up %.2f s" % warm)
    rng = np.random.default_rng(seed)
    out = {"precision": precision, "md_replicas": replicas, "md_atoms": int(md.n_atoms.sum()), "workers": 2,
           "gemm_tiles": "single-CTA (the server's default: no CTA-pair tiles from concurrent streams)",
           "warmup_s": warm, "loads": []}
    for rate in loads:
        count = max(20, int(rate * seconds))
        arrivals = poisson_arrivals(rate, count, seed=int(rate))
        structs = [reqpool[i] for i in rng.integers(0, len(reqpool), count)]
        _, st = srv.run(structs, arrivals, timeout=3.0 * seconds + 20.0)
        st["offered_rps"] = rate
        out["loads"].append(st)
        log("serving: %g req/s -> p50 %.2f ms p99 %.2f ms (%d requests, %d unfinished)"
            % (rate, st["p50_ms"], st["p99_ms"], st["requests"], st["unfinished"]))
        out["md_counters"] = md.counters()
        if report:
            report(out)
    return out


def child_leg(args):
    """Runs one leg (batch or serving) in this child process and writes its results to
    args.out (after every part, so that a run cut short by its budget still reports)."""
    from quip_gb300 import models as mdl

    def report(obj):
        tmp = args.out + ".tmp"
        with open(tmp, "w") as f:
            json.dump(obj, f)
        os.replace(tmp, args.out)

    t0 = time.perf_counter()
    pool = mdl.triclinic_batch(1024, n_min=8, n_max=2048, seed=7, workers=min(16, os.cpu_count() or 1))
    log("%s: 1024 triclinic structures generated in %.1f s" % (args.leg, time.perf_counter() - t0))
    if args.leg == "batch":
        report(measure_batch(args.model, args.precision, pool))
    else:
        measure_serving(args.model, args.precision, pool, [float(x) for x in args.serving_loads.split(",")],
                        args.serving_seconds, report=report)
    return 0


def run_child(leg, args, model_path, tmp, budget_s):
    """The leg in a child process (its own CUDA context), killed with its process group
    when `budget_s` runs out; returns what it reported, with the wall time."""
    if budget_s < 30:
        return {"skipped": "budget", "budget_s": budget_s}
    out = os.path.join(tmp, leg + ".json")
    cmd = [sys.executable, os.path.abspath(__file__), "--leg", leg, "--model", model_path, "--out", out,
           "--precision", args.precision, "--serving-loads", args.serving_loads,
           "--serving-seconds", str(args.serving_seconds)]
    log("%s: child process, budget %.0f s" % (leg, budget_s))
    t0 = time.perf_counter()
    p = subprocess.Popen(cmd, stdout=subprocess.DEVNULL, start_new_session=True)
    status = "ok"
    try:
        rc = p.wait(timeout=budget_s)
        if rc != 0:
            status = "exit %d" % rc
    except subprocess.TimeoutExpired:
        status = "killed at its budget"
        try:
            os.killpg(p.pid, signal.SIGKILL)
        except OSError:
            pass
        p.wait()
    wall = time.perf_counter() - t0
    res = {}
    if os.path.exists(out):
        try:
            res = json.load(open(out))
        except Exception as e:
            res = {"error": "unreadable result: %s" % str(e)[:80]}
    res["leg_status"] = status
    res["leg_wall_s"] = wall
    res["leg_budget_s"] = budget_s
    log("%s: %s after %.1f s" % (leg, status, wall))
    return res


# ---------------------------------------------------------------- reference arm
def reference_arm(args, w):
    from oracle import oracle

    def oracle_descriptor_fn(desc, a):
        return oracle.soap(desc, a.positions, a.numbers, a.lattice, a.pbc)

    tmp = tempfile.mkdtemp(prefix="gapref")
    log("reference: structure and model")
    at = make_structure(w)
    path = make_model(w, tmp, oracle_descriptor_fn)
    full = len(at) * w["M"] * w["n_max"] <= 4096 * 2000 * 8
    sample = None if full else CPU_SAMPLE
    log("reference: timing the oracle (%s)" % ("all centres" if full else "%d sampled centres" % CPU_SAMPLE))
    cb = cpu_reference(w, at, path, args.steps, args.warmup, sample)
    cpu = {k: cb[k] for k in CPU_KEYS if k in cb}
    cpu["cpu_model"] = cpu_model()
    # one thread, on fewer centres (the per-centre cost is what scales)
    st = cpu_reference(w, at, path, 3, 1, None if full else 16, nthreads=1)
    cpu["single_thread"] = {k: st[k] for k in CPU_KEYS if k in st}
    if args.cpu_full and not full:
        log("reference: one oracle call over all %d centres" % len(at))
        t0 = time.perf_counter()
        oracle.OracleModel.from_xml(path).calc(at.positions, at.numbers, at.lattice, [1, 1, 1], nthreads=os.cpu_count())
        tf = time.perf_counter() - t0
        cpu["full_structure"] = {"seconds": tf, "value": len(at) / tf, "extrapolated_value": cb["value"],
                                 "ratio_extrapolated_to_full": cb["value"] / (len(at) / tf)}
    line = {"impl": "reference", "metric": METRIC, "value": cb["value"], "unit": "atom-evals/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * cb["seconds_per_sample"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded structures, random GAP model)",
            "config": {"workload": args.workload, "precision": "fp64", "atoms": len(at), "sparse_points": w["M"]},
            "cpu_baseline": cpu,
            "e2e": {"value": cb["value"], "unit": "atom-evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------- the GPU arm
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="sic32768", choices=sorted(WORKLOADS))
    ap.add_argument("--precision", default="fp16", choices=["fp64", "bf16x3", "tf32", "fp16"])
    ap.add_argument("--budget", type=float, default=960.0,
                    help="wall-clock seconds for the whole run; the batch and serving legs get what is left")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64-compare", action="store_true", help="skip the FP64 comparison run (profiling)")
    ap.add_argument("--no-forms", action="store_true", help="skip the other mixed forms")
    ap.add_argument("--no-batch", action="store_true", help="skip the 1024-structure batched measurement")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving measurement")
    ap.add_argument("--serving-loads", default="500,1500,4000", help="offered loads (requests/s)")
    ap.add_argument("--serving-seconds", type=float, default=3.0)
    ap.add_argument("--gemm-pairs", type=int, default=1, choices=[0, 1, 2],
                    help="CTA-pair GEMM tiles: 0 off, 1 autotuner candidates, 2 only")
    ap.add_argument("--no-autotune", action="store_true",
                    help="GEMM tiles by the built-in rule instead of timing the candidates (profiling)")
    ap.add_argument("--cpu-full", action="store_true", help="reference arm: also one oracle call over all centres")
    # internal: one leg in a child process
    ap.add_argument("--leg", choices=["batch", "serving"], help=argparse.SUPPRESS)
    ap.add_argument("--model", help=argparse.SUPPRESS)
    ap.add_argument("--out", help=argparse.SUPPRESS)
    args = ap.parse_args()
    if args.leg:
        return child_leg(args)
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    w = dict(WORKLOADS[args.workload], name=args.workload)
    warmup = max(3, args.warmup)
    args.warmup = warmup

    if args.impl == "reference":
        if rank != 0:
            return 0
        return reference_arm(args, w)

    deadline = T_START + args.budget
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
        dist.init_process_group("nccl")
    from quip_gb300 import _lib, models
    from quip_gb300.potential import Potential

    tmp = tempfile.mkdtemp(prefix="gapbench")
    log("structure %s" % args.workload)
    at = make_structure(w)
    log("model (sparse points from GPU FP64 descriptors)")
    path = make_model(w, tmp, models.bootstrap_descriptor_fn("fp64"))
    n = len(at)
    lat = np.asfortranarray(at.lattice).ravel(order="F").copy()
    pbc = np.ones(3, np.int32)
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    d_pos = torch.tensor(at.positions, dtype=torch.float64, device="cuda").contiguous()
    d_Z = torch.tensor(at.numbers, dtype=torch.int32, device="cuda")

    def device_run(pot, steps, warm, timed_clocks=None):
        L = pot._L
        _lib.check(L.gapgpu_context_set_stream(pot._ctx, _lib.ctypes.c_void_p(stream.cuda_stream)))
        d_E = torch.zeros(1, dtype=torch.float64, device="cuda")
        d_F = torch.zeros((n, 3), dtype=torch.float64, device="cuda")
        d_V = torch.zeros(9, dtype=torch.float64, device="cuda")

        def step():
            _lib.check(L.gapgpu_calc_device(pot._ctx, n, d_pos.data_ptr(), d_Z.data_ptr(), _lib.ptr(lat), _lib.ptr(pbc),
                                            d_E.data_ptr(), d_F.data_ptr(), d_V.data_ptr()))

        for _ in range(warm):
            step()
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        stage = np.zeros(len(STAGES))
        launches = 0
        with timed_clocks if timed_clocks is not None else contextlib.nullcontext():
            for k in range(steps):
                flush.zero_()
                evs[k][0].record(stream)
                step()
                evs[k][1].record(stream)
                stage += np.array(list(pot.timings().values()))
                launches += pot.launches()
            torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        ms = [a.elapsed_time(b) for a, b in evs]
        return dict(t=sum(ms) / 1e3, ms=ms, stage=stage / steps, launches=launches, E=float(d_E.item()),
                    F=d_F.cpu().numpy(), V=d_V.cpu().numpy().reshape(3, 3, order="F"))

    def stage_dict(stage):
        return dict(zip(STAGES, [round(float(x), 4) for x in stage]))

    # ---- headline: device-resident timing
    log("headline %s: %d warm-up + %d timed steps of %d atoms" % (args.precision, warmup, args.steps, n))
    pot = Potential(param_filename=path, precision=args.precision)
    pot.set_option("pairs", args.gemm_pairs)
    if args.no_autotune:
        pot.set_option("autotune", 0)
    clk = clock_sampler(os.path.join(tmp, "clocks.csv"))
    # NVML samples only the timed steps; nvidia-smi needs its start-up time, so it runs
    # from before the warm-up
    nvml = isinstance(clk, NvmlClocks)
    with contextlib.nullcontext() if nvml else clk:
        t_wall0 = time.perf_counter()
        run = device_run(pot, args.steps, warmup, timed_clocks=clk if nvml else None)
        t_wall = time.perf_counter() - t_wall0
    t_dev = max_over_ranks(run["t"])
    value = world * n * args.steps / t_dev
    stage = run["stage"]
    log("headline: %.3f ms/step, %.4g atom-evals/s" % (1e3 * t_dev / args.steps, value))

    # ---- end to end through the public host API (gapgpu_calc) with pinned buffers
    L = pot._L
    pin_pos = torch.tensor(at.positions, dtype=torch.float64).pin_memory()
    pin_Z = torch.tensor(at.numbers, dtype=torch.int32).pin_memory()
    pin_F = torch.zeros((n, 3), dtype=torch.float64).pin_memory()
    pin_V = torch.zeros(9, dtype=torch.float64).pin_memory()
    pin_E = torch.zeros(1, dtype=torch.float64).pin_memory()

    def e2e_step():
        _lib.check(L.gapgpu_calc(pot._ctx, n, pin_pos.data_ptr(), pin_Z.data_ptr(), _lib.ptr(lat), _lib.ptr(pbc), None,
                                 pin_E.data_ptr(), None, pin_F.data_ptr(), pin_V.data_ptr(), None, b""))

    for _ in range(2):
        e2e_step()
    e2e_ms = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e2e_step()
        e2e_ms.append(1e3 * (time.perf_counter() - t0))
    e2e_value = world * n * args.steps / max_over_ranks(sum(e2e_ms) / 1e3)
    log("e2e: %.3f ms/step" % (sum(e2e_ms) / len(e2e_ms)))

    extras = rank == 0 and world == 1   # the comparisons and legs run on a single GPU only

    # ---- the plain FP64 path on the same structure: throughput and each mixed form's error
    r64 = fp64 = None

    def errors_vs(r, ref):
        return {"force_max_eV_per_A": float(np.abs(r["F"] - ref["F"]).max()),
                "force_rms_eV_per_A": float(np.sqrt(np.mean((r["F"] - ref["F"]) ** 2))),
                "energy_per_atom_eV": abs(r["E"] - ref["E"]) / n,
                "virial_max_eV": float(np.abs(r["V"] - ref["V"]).max())}

    if extras and args.precision != "fp64" and not args.no_fp64_compare:
        log("fp64 comparison run")
        pot64 = Potential(param_filename=path, precision="fp64")
        r64 = device_run(pot64, 2, 1)
        fp64 = {"value": n * 2 / r64["t"], "unit": "atom-evals/s", "ms_per_step": 1e3 * r64["t"] / 2,
                "stage_ms": stage_dict(r64["stage"]), "mixed_speedup": value / (n * 2 / r64["t"]),
                "error_vs_fp64": errors_vs(run, r64), "force_max_abs_eV_per_A": float(np.abs(r64["F"]).max())}
        del pot64
        log("fp64: %.1f ms/step" % fp64["ms_per_step"])

    # ---- the other mixed forms on the same structure
    forms = {}
    form_pots = {args.precision: pot}
    if extras and args.precision != "fp64" and not args.no_forms:
        for prec in ("fp16", "tf32", "bf16x3"):
            if prec == args.precision or time.perf_counter() > deadline - 420:
                continue
            log("form %s" % prec)
            p = Potential(param_filename=path, precision=prec)
            p.set_option("pairs", args.gemm_pairs)
            k = max(3, min(args.steps, 5))
            r = device_run(p, k, 2)
            forms[prec] = {"arithmetic": PRECISION_TEXT[prec], "value": n * k / r["t"], "unit": "atom-evals/s",
                           "ms_per_step": 1e3 * r["t"] / k, "steps": k, "stage_ms": stage_dict(r["stage"])}
            if r64 is not None:
                forms[prec]["error_vs_fp64"] = errors_vs(r, r64)
                forms[prec]["speedup_vs_fp64"] = forms[prec]["value"] / fp64["value"]
            form_pots[prec] = p
            log("form %s: %.3f ms/step" % (prec, forms[prec]["ms_per_step"]))

    # ---- neighbour statistics for the algorithmic counts
    off, j, sh = pot.neighbours(at, w["cutoff"])
    d = at.positions[j] - np.repeat(at.positions, np.diff(off), axis=0) + (at.lattice @ sh.T).T
    nu = float(np.sum(np.linalg.norm(d, axis=1) < w["cutoff"])) / n
    flops_atom, gemm_atom = algorithmic_flops(w, nu)
    sflops = stage_flops(w, nu)
    pk = peaks()

    # ---- ceilings: cuBLAS TF32 and the FP32 FMA rate, measured here
    tf32_peak = fp32_peak = None
    if extras:
        torch.backends.cuda.matmul.allow_tf32 = True
        a = torch.randn(8192, 8192, device="cuda")
        b = torch.randn(8192, 8192, device="cuda")
        for _ in range(3):
            a @ b
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(10):
            a @ b
        e1.record()
        torch.cuda.synchronize()
        tf32_peak = 10 * 2 * 8192 ** 3 / (e0.elapsed_time(e1) / 1e3) / 1e12
        del a, b
        v = _lib.ctypes.c_double()
        _lib.check(L.gapgpu_probe_fp32_rate(pot._ctx, _lib.ctypes.byref(v)))
        fp32_peak = v.value
        log("ceilings: cuBLAS TF32 %.0f TFLOP/s, FP32 FMA %.1f TFLOP/s" % (tf32_peak, fp32_peak))

    def gemm_ceiling(prec):
        """The rate the two kernel GEMMs of this form can reach, and where it comes from."""
        if prec == "fp16":
            return pk["bf16_tflops"], "of measured: bf16 burst %.1f TF/s (MEASURED_PEAKS.json; FP16 shares the rate)" % (
                pk["bf16_tflops"])
        if prec == "bf16x3":
            return pk["bf16_tflops"] / 3, "of measured: bf16 burst %.1f TF/s / 3 (three split-BF16 products)" % (
                pk["bf16_tflops"])
        if prec == "tf32":
            return tf32_peak, "of measured: cuBLAS TF32 8192^3 in this run"
        return None, None

    def roofline_of(prec, stage_ms):
        peak, note = gemm_ceiling(prec)
        gemm_ms = stage_ms[2] if isinstance(stage_ms, (list, np.ndarray)) else stage_ms["gemm"]
        ach = n * gemm_atom / (gemm_ms / 1e3) / 1e12 if gemm_ms > 0 else None
        return {"bound": "tensor", "achieved": ach, "peak": peak, "unit": "TFLOP/s",
                "frac": (ach / peak) if (ach and peak) else None, "peak_source": note,
                "gemm_ms_per_step": gemm_ms, "gemm_flops_per_atom": gemm_atom,
                "tensor_pipe_flops_per_atom": gemm_atom * (3.0 if prec == "bf16x3" else 1.0)}

    roofline = None
    stage_roofline = {}
    if args.precision != "fp64":
        roofline = roofline_of(args.precision, stage)
        gemm2_f16 = any(t.startswith("f16 store") for t in _lib.tuning_report().splitlines())
        gemm1_f16 = any(t.startswith("f16 kernel") for t in _lib.tuning_report().splitlines())
        roofline["kernel"] = ("sparse-GP kernel GEMMs, both launches (tcgen05, tiles chosen by the autotuner): "
                              "K = Q X^T with the fused kernel epilogue, G = W X")
        # DRAM bytes of the two GEMM launches from the ncu capture of the 8192-atom case with
        # this model (CTA-pair tiles, both GEMMs in FP16: 93+93 MB and 176+31 MB read+written),
        # scaled by the row count: the operand re-reads and the W/G traffic grow with the rows
        roofline["traffic"] = ((93 + 93 + 176 + 31) * 1e6 * n / 8192
                               if args.precision == "fp16" and w["kind"] == "sic" and gemm1_f16 and gemm2_f16 else None)
        roofline["traffic_note"] = ("DRAM bytes per step of the two GEMM launches, ncu capture at 8192 atoms scaled by "
                                    "the row count" if roofline["traffic"] else None)
        for prec, f in forms.items():
            f["roofline"] = roofline_of(prec, f["stage_ms"])
        if fp32_peak:
            for key in ("soap_fwd", "soap_bwd"):
                ms = stage[STAGES.index(key)]
                ach = n * sflops[key] / (ms / 1e3) / 1e12 if ms > 0 else None
                stage_roofline[key] = {"bound": "fp32 issue", "achieved": ach, "peak": fp32_peak, "unit": "TFLOP/s",
                                       "frac": ach / fp32_peak if ach else None, "ms_per_step": ms,
                                       "flops_per_centre": sflops[key],
                                       "peak_source": "FP32 FMA-loop kernel measured in this run "
                                                      "(gapgpu_probe_fp32_rate)"}
    else:
        # the plain path: its FP64 SIMT GEMMs against cuBLAS DGEMM measured here
        a = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
        b = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
        for _ in range(2):
            a @ b
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(5):
            a @ b
        e1.record()
        torch.cuda.synchronize()
        peak = 5 * 2 * 4096 ** 3 / (e0.elapsed_time(e1) / 1e3) / 1e12
        ach = n * gemm_atom / (stage[2] / 1e3) / 1e12 if stage[2] > 0 else None
        roofline = {"bound": "fp64", "kernel": "sparse-GP kernel GEMMs (FP64 SIMT)", "achieved": ach, "peak": peak,
                    "unit": "TFLOP/s", "frac": ach / peak if ach else None, "traffic": None,
                    "peak_source": "cuBLAS DGEMM 4096^3 measured in this run"}

    # ---- CPU baseline: the oracle on a sample of centres, and each form's error against it
    cpu = None
    if extras and not args.no_cpu_baseline:
        sample = None if n * w["M"] <= 4096 * 2000 else CPU_SAMPLE
        log("cpu baseline (oracle, %s)" % ("all centres" if sample is None else "%d sampled centres" % sample))
        try:
            kept = {}
            cb = cpu_reference(w, at, path, 1, 0, sample, keep=kept)
            cpu = {k: cb[k] for k in CPU_KEYS if k in cb}
            cpu["cpu_model"] = cpu_model()
            o, mask = kept["result"], kept["mask"]
            nc = sample or n
            errs = {}
            for prec, p in form_pots.items():
                g = p.calc(at, atom_mask=mask)
                errs[prec] = {"centres": nc, "force_max_eV_per_A": float(np.abs(g["force"] - o["force"]).max()),
                              "energy_per_centre_eV": abs(g["energy"] - o["energy"]) / nc,
                              "virial_max_eV": float(np.abs(g["virial"] - o["virial"]).max())}
            cpu["sampled_error_vs_oracle"] = errs[args.precision]
            for prec, f in forms.items():
                f["sampled_error_vs_oracle"] = errs[prec]
        except Exception as e:
            cpu = {"value": None, "error": str(e)[:160]}
    form_pots = None   # the forms' contexts and models are freed before the child legs

    # ---- batch and serving, each in a child process with what is left of the budget
    batch = serving = None
    if extras and w["kind"] == "sic":
        if not args.no_batch:
            batch = run_child("batch", args, path, tmp, min(300.0, deadline - time.perf_counter() - 330))
        if not args.no_serving:
            serving = run_child("serving", args, path, tmp, min(300.0, deadline - time.perf_counter() - 20))

    if rank == 0:
        h2d = n * 3 * 8 + n * 4
        d2h = 8 + n * 3 * 8 + 9 * 8
        line = {"metric": METRIC, "value": value, "unit": "atom-evals/s", "n_gpus": world, "steps": args.steps,
                "warmup": warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": DTYPE[args.precision],
                "data": "synthetic: seeded structures and a random GAP model (no published dataset for this path)",
                "config": {"workload": args.workload, "precision": args.precision,
                           "arithmetic": PRECISION_TEXT[args.precision], "atoms": n, "sparse_points": w["M"],
                           "soap": "n_max=%d l_max=%d rc=%g species=%s" % (w["n_max"], w["l_max"], w["cutoff"],
                                                                           list(w["species"])),
                           "mean_neighbours": nu, "l2": "256 MB flush between timed steps",
                           "parallelism": "replicas" if world > 1 else "single GPU"},
                "stage_ms": stage_dict(stage), "fp64": fp64, "forms": forms or None, "roofline": roofline,
                "stage_roofline": stage_roofline or None, "cpu_baseline": cpu,
                "e2e": {"value": e2e_value, "unit": "atom-evals/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                        "p50_ms": float(np.percentile(e2e_ms, 50)), "p99_ms": float(np.percentile(e2e_ms, 99))},
                "gpu_launches": int(run["launches"]), "clocks": clk.summary(), "batch": batch, "serving": serving,
                "autotune": _lib.tuning_report().strip().splitlines(), "ceilings": {"tf32_tflops": tf32_peak,
                                                                                  "fp32_fma_tflops": fp32_peak},
                "algorithmic_flops_per_atom": flops_atom, "wall_s": t_wall,
                "bench_wall_s": time.perf_counter() - T_START}
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

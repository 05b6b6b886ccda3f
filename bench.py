"""Benchmark: GRI-Mech 3.0 dense FP64 analytical Jacobians on one GB300.

Headline workload: GRI-Mech 3.0 (53 species, 325 reactions), 1,048,576
seeded synthetic states (T ~ U(800, 2200) K, P log-uniform 1-25 atm,
X ~ Dirichlet(0.5) floored at 1e-12, V = 1 m^3), constant pressure, F data
order, dense 54 x 54 Jacobian.  One step = one Jacobian evaluation of all
states (pjg_jacobian).  Inputs (453 MB) and outputs (24.5 GB) are larger than
L2, so no flush is needed between steps.

The same JSON line carries, under ``configs``, the other benchmark
configurations, each timed on the device with its roofline, a CPU baseline on
the same host and a sampled parity check against the oracle: H2/O2 dense
Jacobian and species rates (65,536 states, C order), GRI-Mech 3.0 species
rates and sparse Jacobians (CCS in F order, CRS in C order, 1,048,576
states), the seeded 500-species synthetic mechanism's sparse CRS Jacobian
(131,072 states) and the J^T v kernel behind the torch wdot
autograd.Function (262,144 states).  The headline output itself is checked
too (``parity``): states at both ends, around every launch boundary and at
random, each compared whole, so element offsets above 2^31 are covered.

Other single configurations: ``--mech h2o2|synthetic500``, ``--format
sparse``, ``--order C``, ``--kernel rates|vjp``, ``--states N``.

``--gpus N``: one process per GPU (torchrun, or spawned here when torchrun did
not start this process), each evaluating its own 1,048,576 states (weak
scaling); rank 0 prints the line.  ``--impl reference`` times the reference's
CPU implementation of the headline on the host cores instead, with the same
``config``: the shim-compiled shipped GRI or H2/O2 kernels in oracle/_ref
when they load here, else the C oracle (the CPU restatement of the
reference) with OpenMP on all cores.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
import importlib  # noqa: E402

PKG = "pyjac-v2_gb300"
METRIC = "GRI-30 FP64 Jacobians/s"
UNIT = "Jacobians/s"
# per --kernel: metric, unit, evaluation kernel
KERNELS = {
    "jacobian": (METRIC, UNIT, "eval_kernel<1> (fused Jacobian)"),
    "rates": ("GRI-30 FP64 species-rate evaluations/s", "states/s", "eval_kernel<0> (species rates)"),
    "vjp": ("GRI-30 FP64 J^T v products/s", "states/s", "eval_kernel<2> (J^T v)"),
}
KIND = {"rates": 0, "jacobian": 1, "vjp": 2}
# executed FP64 instruction / DRAM counts per state (ncu captures, profiles/)
NCU_COUNTS = os.path.join(ROOT, "profiles", "gri30_kernel_counts.json")
# algorithmic FP64 operations per state of the reference's formulation
# (counted by the oracle: oracle/count_flops.py)
OP_COUNTS = os.path.join(ROOT, "data", "fp64_op_counts.json")

# --mech: the benchmark configurations' mechanisms, their label and the
# reference's shipped kernels for the CPU baseline (None: the C oracle port)
MECHS = {
    "gri30": ("GRI-30", "ch4", "grimech30 (53 species, 325 reactions)"),
    "h2o2": ("H2/O2", "h2o2", "h2o2 (9 species, 28 reactions)"),
    "synthetic500": ("synthetic-500", None, "seeded synthetic (500 species, 2,500 reactions)"),
}

# The benchmark configurations measured beside the headline (key: mechanism,
# kernel, Jacobian format, order, states, CPU-baseline states per step).
CONFIGS = [
    ("h2o2_dense_C_65536", "h2o2", "jacobian", "full", "C", 65536, 262144),
    ("h2o2_rates_C_65536", "h2o2", "rates", "full", "C", 65536, 1048576),
    ("gri30_rates_F_1M", "gri30", "rates", "full", "F", 1 << 20, 262144),
    ("gri30_sparse_F_1M", "gri30", "jacobian", "sparse", "F", 1 << 20, None),
    ("gri30_sparse_C_1M", "gri30", "jacobian", "sparse", "C", 1 << 20, None),
    ("synthetic500_sparse_C_131072", "synthetic500", "jacobian", "sparse", "C", 131072, 2048),
    ("vjp_gri30_262144", "gri30", "vjp", "full", "F", 262144, 32768),
]


def pkg(sub=None):
    return importlib.import_module(PKG + ("." + sub if sub else ""))


def oracle_mod():
    p = os.path.join(ROOT, "oracle")
    if p not in sys.path:
        sys.path.insert(0, p)
    return importlib.import_module("oracle")


def alg_bytes_per_state(nn, n_out, n_in=None):
    """Algorithmic HBM bytes per state: read phi (NN) + param (+ v for J^T v),
    write n_out values."""
    return 8 * (nn + 1 if n_in is None else n_in) + 8 * n_out


def io_sizes(mech, kernel, fmt):
    """(values written, values read) per state."""
    nn = mech.nn
    if kernel == "jacobian":
        return (nn * nn if fmt == "full" else mech.jac_nnz()), nn + 1
    return nn, (nn + 1 if kernel == "rates" else 2 * nn + 1)


_mech_cache = {}


def load_mech(name, jac_type="exact"):
    key = (name, jac_type)
    if key in _mech_cache:
        return _mech_cache[key]
    if name == "gri30":
        m = pkg().load_mechanism(os.path.join(ROOT, "data", "grimech30.inp"),
                                 os.path.join(ROOT, "data", "thermo30.dat"), jac_type=jac_type)
    elif name == "h2o2":
        m = pkg().load_mechanism(os.path.join(ROOT, "data", "h2o2.inp"), jac_type=jac_type)
    else:
        import tempfile
        path = os.path.join(tempfile.gettempdir(), "pyjac_gb300_synthetic500_seed0.inp")
        if not os.path.exists(path):
            pkg("mech.synthetic").write(path + ".tmp")  # defaults: 500 species, 2,500 reactions
            os.replace(path + ".tmp", path)
        m = pkg().load_mechanism(path, jac_type=jac_type)
    _mech_cache[key] = m
    return m


def read_json(path):
    if not os.path.exists(path):
        return {}
    with open(path) as fh:
        return json.load(fh)


def hbm_peak():
    d = read_json(os.path.join(ROOT, "MEASURED_PEAKS.json"))
    if d.get("hbm_gbs"):
        return float(d["hbm_gbs"]), "measured (MEASURED_PEAKS.json)"
    return 6800.0, "fallback"


class ClockSampler(object):
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


# ------------------------------------------------------------------ CPU baseline

def cpu_reference_run(mech, n_sample, steps, seed=1, warmup=1, mech_name="gri30",
                      kernel="jacobian"):
    """Time the reference's CPU implementation of `kernel` on n_sample states
    per step, all host threads: (baseline dict, seconds per step)."""
    orc = oracle_mod()
    states = pkg("states")
    P, phi = states.draw_states(mech.n_species, n_sample, seed=seed, x_floor=1e-12)
    threads = cpu_threads()
    kind, fn, desc = None, None, None
    label, shipped, _ = MECHS[mech_name]
    if shipped and kernel != "vjp" and orc.RefKernels.available(shipped):
        try:
            ref = orc.RefKernels(shipped)
            phiF = np.ascontiguousarray(phi.T)
            kind = "reference"
            if kernel == "jacobian":
                desc = ("reference shipped %s kernels (examples/opencl/%s, %s Jacobian, F order), "
                        "shim-compiled" % (label, shipped, "sparse CCS" if shipped == "ch4" else "dense"))

                def fn():
                    ref.jacobian_F(P, phiF, nthreads=threads)
            else:
                desc = ("reference shipped %s species_rates kernel (examples/opencl/%s, F order), "
                        "shim-compiled" % (label, shipped))

                def fn():
                    ref.species_rates_F(P, phiF, nthreads=threads)
        except OSError:
            kind = None
    if kind is None:
        o = orc.Oracle(mech)
        kind = "port"
        if kernel == "jacobian":
            desc = "C oracle (CPU restatement of the reference), dense Jacobian, OpenMP"

            def fn():
                o.jacobian(P, phi, conp=True, nthreads=threads)
        elif kernel == "rates":
            desc = "C oracle (CPU restatement of the reference), species rates, OpenMP"

            def fn():
                o.species_rates(P, phi, conp=True, nthreads=threads)
        else:
            v = np.random.default_rng(seed + 1).standard_normal(phi.shape)
            desc = ("C oracle (CPU restatement of the reference): dense Jacobian, OpenMP, then "
                    "J^T v by numpy (the reference has no J^T v)")

            def fn():
                J = o.jacobian(P, phi, conp=True, nthreads=threads)
                np.einsum("nrc,nr->nc", J, v)
    for _ in range(max(1, warmup)):  # untimed calls first (the reference's main times its second)
        fn()
    ts = []
    for _ in range(max(1, steps)):
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    sec = float(np.mean(ts))
    unit = UNIT if kernel == "jacobian" else "states/s"
    return {"value": n_sample / sec, "unit": unit, "cores": threads, "kind": kind,
            "sample": "%d %s states per step, %s" % (n_sample, label, desc)}, sec


# ------------------------------------------------------------------ parity

def sample_states(n, chunk, rng, n_random=512, n_end=64):
    """Sampled state indices: both ends, around every launch boundary, and at
    random."""
    idx = set(range(min(n, n_end))) | set(range(max(0, n - n_end), n))
    if chunk and chunk < n:
        for b in range(chunk, n, chunk):
            idx |= set(range(max(0, b - 2), min(n, b + 2)))
    idx |= set(rng.choice(n, size=min(n, n_random), replace=False).tolist())
    return np.array(sorted(idx), dtype=np.int64)


def _to_dense(vals, ptr, ind, nn, order):
    """Sparse values (m, nnz) in CRS ('C') or CCS ('F') order -> dense (m, nn, nn)."""
    m = vals.shape[0]
    J = np.zeros((m, nn, nn))
    for a in range(nn):
        for p in range(ptr[a], ptr[a + 1]):
            if order == "C":
                J[:, a, ind[p]] = vals[:, p]
            else:
                J[:, ind[p], a] = vals[:, p]
    return J


def gather_output(out, kernel, fmt, order, n, nn, nnz, idx):
    """The sampled states' outputs from a device output array, as numpy:
    (m, nn, nn) dense / (m, nnz) sparse for the Jacobian, (m, nn) otherwise."""
    import torch
    t = torch.from_numpy(idx).to(out.device)
    if kernel != "jacobian":
        v = out.reshape(nn, n)[:, t].T if order == "F" else out.reshape(n, nn)[t]
    elif fmt == "full":
        v = out.reshape(nn, nn, n)[:, :, t].permute(2, 1, 0) if order == "F" \
            else out.reshape(n, nn, nn)[t]
    else:
        v = out.reshape(nnz, n)[:, t].T if order == "F" else out.reshape(n, nnz)[t]
    return v.contiguous().cpu().numpy()


def parity_check(mech, ev, kernel, fmt, order, P, phi, out, tP, tphi, tv=None, chunk=None,
                 seed=99, n_random=512, n_end=64):
    """Compare a sample of a device output with the oracle.  P, phi: host
    states (phi in C order); out: the device output of all n states in
    `order`/`fmt`.  Rates are re-evaluated on the device for the same states
    (same order) and compared too."""
    import torch
    orc = oracle_mod()
    n, nn = P.shape[0], mech.nn
    idx = sample_states(n, chunk, np.random.default_rng(seed), n_random, n_end)
    o = orc.Oracle(mech)
    Ps, phis = P[idx], phi[idx]
    thr = cpu_threads()
    res = {"n_checked": int(idx.size), "sample": "first/last %d, +-2 around each launch boundary "
           "(%s states per launch), %d random" % (n_end, chunk, n_random)}
    # species rates of the same states from the device, in the run's order
    d = ev.species_rates(tP, tphi, order=order, conp=True)
    dg = gather_output(d, "rates", fmt, order, n, nn, 0, idx)
    del d
    dref = o.species_rates(Ps, phis, nthreads=thr)
    scale = o.rates_scale(Ps, phis, nthreads=thr)
    res["rates_max_rel"] = float((np.abs(dg - dref) / np.maximum(np.abs(dref), 1e-300)).max())
    diff = np.abs(dg - dref)
    res["rates_max_rel_cancellation_scaled"] = float(
        (diff / np.maximum(np.abs(dref) + scale, 1e-300)).max())
    well = (np.abs(dref) >= 1e-3 * scale) & (dref != 0)
    res["rates_max_rel_well_conditioned"] = float((diff[well] / np.abs(dref[well])).max()) \
        if well.any() else 0.0
    res["rates_bar"] = "1e-10 relative to |value| + cancellation scale (the same sums in absolute " \
                       "values) for every entry, and 1e-10 relative to |value| for entries of at " \
                       "least 1e-3 of their scale"
    res["rates_pass"] = bool(res["rates_max_rel_cancellation_scaled"] <= 1e-10 and
                             res["rates_max_rel_well_conditioned"] <= 1e-10)
    if kernel == "vjp":
        got = gather_output(out, "vjp", fmt, order, n, nn, 0, idx)
        J = o.jacobian(Ps, phis, nthreads=thr)
        v = gather_output(tv, "vjp", fmt, order, n, nn, 0, idx)
        ref = np.einsum("nrc,nr->nc", J, v)
        sc = np.einsum("nrc,nr->nc", np.abs(J), np.abs(v))
        res["vjp_max_rel_to_abs_product"] = float((np.abs(got - ref) / np.maximum(sc, 1e-300)).max())
        res["vjp_pass"] = bool(res["vjp_max_rel_to_abs_product"] <= 1e-10)
        return res
    if kernel == "rates":
        return res
    Jref = o.jacobian(Ps, phis, nthreads=thr)
    g = gather_output(out, "jacobian", fmt, order, n, nn, mech.jac_nnz(), idx)
    if fmt == "sparse":
        ptr, ind = mech.pattern(order)
        g = _to_dense(g, ptr, ind, nn, order)
        mask = _to_dense(np.ones((1, len(ind))), ptr, ind, nn, order)[0] > 0
    else:
        mask = np.ones((nn, nn), dtype=bool)
    rowmax = np.abs(Jref).max(axis=2, keepdims=True)
    rowmax[rowmax == 0] = 1.0
    err = np.abs(g - Jref) * mask
    res["jac_max_row_rel"] = float((err / rowmax).max())
    well = (np.abs(Jref) >= 1e-6 * rowmax) & mask
    rel = err[well] / np.abs(Jref[well])
    res["jac_max_elem_rel_well_conditioned"] = float(rel.max()) if rel.size else 0.0
    res["jac_frac_well_conditioned_within_1e-8"] = float((rel <= 1e-8).mean()) if rel.size else 1.0
    res["jac_entries_well_conditioned"] = int(well.sum())
    res["jac_bar"] = "1e-8 relative to the row's largest entry; the element-wise error is reported " \
                     "over entries of at least 1e-6 of their row's largest"
    res["jac_pass"] = bool(res["jac_max_row_rel"] <= 1e-8)
    if fmt == "full" and order == "F":
        res["max_elem_offset_checked"] = int(idx.max() + n * (nn - 1) + n * nn * (nn - 1))
    elif fmt == "full":
        res["max_elem_offset_checked"] = int(idx.max() * nn * nn + nn * nn - 1)
    return res


# ------------------------------------------------------------------ device timing

def timed_steps(step, steps, warmup, stream):
    """Run step() warmup times, then time `steps` calls with CUDA events on
    `stream`; also the evaluation kernels' own time (pjg_profile_*) and the
    number of this library's launches.  Returns (ms total, eval launches,
    eval ms, launches)."""
    import torch
    lib = pkg("_lib")
    for _ in range(max(3, warmup)):
        step()
    torch.cuda.synchronize()
    launches0 = lib.launch_count()
    lib.profile_begin()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    n_eval, eval_ms = lib.profile_end()
    return e0.elapsed_time(e1), n_eval, eval_ms, lib.launch_count() - launches0


def fp64_roofline(mech_name, kernel, fmt, order, krate, fp64_peak):
    """FP64 roofline of an evaluation kernel running at krate states/s:
    algorithmic flops from the oracle's operation counter, executed FP64
    instructions (ncu) where a capture of this configuration exists."""
    ops = read_json(OP_COUNTS).get("mechanisms", {}).get(mech_name, {}).get(kernel)
    out = {"peak": fp64_peak, "unit": "TFLOP/s",
           "peak_source": "measured DFMA probe (pjg_fp64_peak)"}
    if ops:
        fl = ops["flops"]
        out.update({"achieved": fl * krate / 1e12, "frac": fl * krate / 1e12 / fp64_peak,
                    "alg_flops_per_state": fl,
                    "transcendentals_per_state": {k: ops[k] for k in ("exp", "log", "log10", "pow")},
                    "minmax_per_state": ops["minmax"],
                    "flops_source": "oracle op counter (data/fp64_op_counts.json): add + mul + "
                                    "div + 2 fma of the reference's formulation; exp/log/pow "
                                    "counted apart, not in flops"})
    key = "%s_%s_%s" % (kernel, fmt if kernel == "jacobian" else "na", order)
    if mech_name != "gri30":
        key = mech_name + "_" + key
    nc = read_json(NCU_COUNTS).get(key)
    if nc:
        ex, ins = nc["fp64_flops_per_state"], nc["fp64_inst_per_state"]
        out.update({"exec_flops_per_state": ex, "exec_inst_per_state": ins,
                    "exec_frac": ex * krate / 1e12 / fp64_peak,
                    "pipe_frac": ins * krate / (fp64_peak * 1e12 / 2),
                    "exec_source": "ncu, %s (profiles/)" % nc.get("case", "")})
        if ops:
            out["exec_over_alg"] = ex / ops["flops"]
    return out


def measure_config(key, mech_name, kernel, fmt, order, n, cpu_sample, dev, steps, warmup,
                   fp64_peak, cpu_cache, seed=1000):
    """One benchmark configuration on the device: throughput with inputs in
    HBM, roofline, CPU baseline on the host and sampled parity."""
    import torch
    api = pkg("api")
    mech = load_mech(mech_name)
    ev = api.Evaluator(mech)
    n_out, n_in = io_sizes(mech, kernel, fmt)
    P, phi = pkg("states").draw_states(mech.n_species, n, seed=seed, x_floor=1e-12)
    x = np.ascontiguousarray(phi.T) if order == "F" else phi
    tP = torch.from_numpy(P).to(dev)
    tphi = torch.from_numpy(x).to(dev)
    out = torch.empty(n * n_out, dtype=torch.float64, device=dev)
    tv = None
    if kernel == "vjp":
        tv = torch.from_numpy(np.random.default_rng(77).standard_normal(x.shape)).to(dev)

    def step():
        if kernel == "jacobian":
            ev.jacobian(tP, tphi, order=order, conp=True, jac_format=fmt, out=out)
        elif kernel == "rates":
            ev.species_rates(tP, tphi, order=order, conp=True, out=out.view(tphi.shape))
        else:
            ev.vjp(tP, tphi, tv, order=order, conp=True, out=out.view(tphi.shape))

    stream = torch.cuda.current_stream(dev)
    ms, n_eval, eval_ms, launches = timed_steps(step, steps, warmup, stream)
    krate = n * steps / (eval_ms * 1e-3)
    bps = alg_bytes_per_state(mech.nn, n_out, n_in)
    peak, src = hbm_peak()
    res = {"workload": "%s %s, %s order, %d states" % (
               MECHS[mech_name][0],
               {"jacobian": ("dense" if fmt == "full" else
                             ("sparse CCS" if order == "F" else "sparse CRS")) + " FP64 Jacobian",
                "rates": "FP64 species rates", "vjp": "FP64 J^T v (v ~ N(0, 1))"}[kernel],
               order, n),
           "value": n * steps / (ms * 1e-3), "unit": UNIT if kernel == "jacobian" else "states/s",
           "ms_per_step": ms / steps, "steps": steps, "gpu_launches": launches,
           "roofline": {"bound": "fp64 pipe",
                        "hbm": {"achieved": bps * krate / 1e9, "peak": peak, "unit": "GB/s",
                                "frac": bps * krate / 1e9 / peak, "alg_bytes_per_state": bps,
                                "peak_source": src},
                        "fp64": fp64_roofline(mech_name, kernel, fmt, order, krate, fp64_peak),
                        "kernel": KERNELS[kernel][2], "eval_ms_per_step": eval_ms / steps}}
    if kernel == "vjp":
        # the same product through the torch autograd.Function (forward rates, backward J^T v)
        tops = pkg("torch_ops")
        tphiC = tphi.T.contiguous() if order == "F" else tphi
        tvC = tv.T.contiguous() if order == "F" else tv

        def ad_step():
            p = tphiC.detach().requires_grad_(True)
            y = tops.wdot(ev, tP, p)
            y.backward(tvC)
        ad_ms, _, _, _ = timed_steps(ad_step, steps, warmup, stream)
        res["autograd_forward_backward_states_per_s"] = n * steps / (ad_ms * 1e-3)
    chunk = pkg("_lib").eval_chunk(ev.handle, KIND[kernel], n, order, 0 if fmt == "full" else 1)
    res["parity"] = parity_check(mech, ev, kernel, fmt, order, P, phi, out, tP, tphi, tv,
                                 chunk=chunk, n_random=512 if mech.nn < 200 else 48,
                                 n_end=64 if mech.nn < 200 else 8)
    del out, tphi, tP, tv
    torch.cuda.empty_cache()
    ck = (mech_name, kernel)
    if ck not in cpu_cache:
        cpu_cache[ck] = cpu_reference_run(mech, cpu_sample or 262144, 2, mech_name=mech_name,
                                          kernel=kernel)[0]
    res["cpu_baseline"] = cpu_cache[ck]
    return res


# ------------------------------------------------------------------ surrogate, implicit step

def surrogate_bench(mech, ev, dev, n_train, epochs, n_eval, log=None, ablation=True):
    """Train the BF16 surrogate on n_train states (Sobolev loss), calibrate
    its error head on held-out states, then report its error against the
    FP64 kernel and the wdot speedup at several tolerances on n_eval fresh
    states (FP64 fallback included in the timed path).  With ablation, the
    same training without the Sobolev term, at equal epochs, beside it."""
    import torch
    sg = pkg("surrogate")
    tols = (1.0, 0.5, 0.3, 1e-1, 1e-2, 1e-3)

    def train(sobolev_weight):
        s = sg.Surrogate(mech, device=dev, evaluator=ev)
        t0 = time.time()
        hist = s.fit(n_train=n_train, epochs=epochs, batch=16384, lr=2e-3, log=log,
                     sobolev_weight=sobolev_weight)
        torch.cuda.synchronize()
        cal = s.calibrate(n=1 << 18, tols=tols)
        return s, hist, time.time() - t0, cal

    s, hist, t_train, cal = train(0.1)
    data = s.make_data(n_eval, seed=4242, sobolev=False)
    P, phi = data["P"], data["phi"]
    stream = torch.cuda.current_stream(dev)

    def timed(fn, reps=3):
        fn()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            r = fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps, r

    t_fp64, _ = timed(lambda: ev.species_rates(P, phi))

    def evaluate(sur):
        t_net, raw = timed(lambda: sur.predict(P, phi))
        y_hat = torch.cat([raw[0][:, :1], raw[0][:, 2:]], dim=1)
        err = sur.rel_error(y_hat, data["y"])
        q = torch.quantile(err[: min(len(err), 1 << 24)].float(),
                           torch.tensor([0.5, 0.9, 0.99], device=dev))
        qmax = torch.quantile(sur.max_rel_error(y_hat, data["y"]).float(),
                              torch.tensor([0.5, 0.9, 0.99], device=dev))
        curve = []
        for tol in tols:
            t_tol, (out, info) = timed(lambda: sur.species_rates(P, phi, tol=tol, return_info=True),
                                       reps=1)
            yo = torch.cat([out[:, :1], out[:, 2:]], dim=1)
            e2 = sur.rel_error(yo, data["y"])
            fb = info["fallback_frac"]
            curve.append({"tol": tol, "ms": t_tol, "fallback_frac": fb,
                          "one_minus_frac_err_below": float((err > tol).float().mean()),
                          "speedup_vs_fp64": t_fp64 / t_tol,
                          "frac_states_within_tol": float((e2 <= tol).float().mean()),
                          "p99_err": float(torch.quantile(e2.float(), 0.99))})
        return t_net, q, qmax, err, curve

    t_net, q, qmax, err, curve = evaluate(s)
    res = {"network": "54 -> 4x256 SiLU -> 53 (+1 error estimate), BF16 weights/activations, "
                      "FP32 accumulate, tcgen05 GEMMs",
           "train_states": n_train, "epochs": epochs, "train_s": t_train,
           "final_value_mse": hist[-1]["value_mse"], "final_sobolev_mse": hist[-1]["sobolev_mse"],
           "eval_states": n_eval, "fp64_rates_ms": t_fp64, "network_ms": t_net,
           "network_speedup_vs_fp64": t_fp64 / t_net,
           "err_median": float(q[0]), "err_p90": float(q[1]), "err_p99": float(q[2]),
           "worst_component_err_median": float(qmax[0]), "worst_component_err_p90": float(qmax[1]),
           "frac_err_below": {str(t): float((err <= t).float().mean()) for t in tols},
           "calibration": {"states": 1 << 18, "precision": 0.99,
                           "rule": "per tolerance, the largest predicted-error threshold whose "
                                   "held-out answered states are 99 % within it",
                           "answered_frac": {str(t): cal[t][1] for t in tols}},
           "with_fallback": curve,
           "error_metric": "per state ||(y_hat - y)/rms|| / ||y/rms|| over dT/dt and the 52 molar "
                           "rates (rms over training states); worst component: "
                           "max_k |y_hat - y| / (|y| + 1e-3 rms_k)"}
    if ablation:
        del s
        torch.cuda.empty_cache()
        s0, hist0, t0_train, _ = train(0.0)
        _, q0, _, err0, curve0 = evaluate(s0)
        res["ablation_no_sobolev"] = {
            "sobolev_weight": 0.0, "epochs": epochs, "train_states": n_train, "train_s": t0_train,
            "final_value_mse": hist0[-1]["value_mse"],
            "err_median": float(q0[0]), "err_p90": float(q0[1]), "err_p99": float(q0[2]),
            "frac_err_below": {str(t): float((err0 <= t).float().mean()) for t in tols},
            "with_fallback": [{k: c[k] for k in ("tol", "fallback_frac", "speedup_vs_fp64")}
                              for c in curve0]}
    return res


STUDY_GRID = ((4, 12, 1 << 20), (4, 12, 1 << 22), (4, 30, 1 << 22), (4, 60, 1 << 22),
              (4, 120, 1 << 22), (8, 30, 1 << 22), (2, 30, 1 << 22))


def surrogate_study(mech, ev, dev, n_eval=1 << 20, grid=STUDY_GRID, log=None):
    """Capacity study of the surrogate: for each (hidden layers, epochs,
    training states) the per-state error on n_eval fresh states, the share of
    states within 1e-1 / 1e-2 / 1e-3, and the same network evaluated with
    FP32 weights and activations (plain torch, a measurement only), which
    separates the BF16 rounding from the fit."""
    import torch
    sg = pkg("surrogate")
    tols = (1e-1, 1e-2, 1e-3)
    rows = []
    for depth, epochs, n_train in grid:
        s = sg.Surrogate(mech, device=dev, evaluator=ev, depth=depth)
        t0 = time.time()
        hist = s.fit(n_train=n_train, epochs=epochs, batch=16384, lr=2e-3, sobolev_weight=0.1)
        torch.cuda.synchronize()
        t_fit = time.time() - t0
        data = s.make_data(n_eval, seed=4242, sobolev=False)
        y_hat, _, X = s.predict_raw(data["P"], data["phi"])
        err = s.rel_error(y_hat, data["y"])
        with torch.no_grad():
            a = X.float()
            for l in range(depth):
                a = torch.nn.functional.silu(a @ s.net.W[l].t() + s.net.b[l])
            y32 = s.untransform((a @ s.net.W[-1].t() + s.net.b[-1])[:, :sg.NOUT])
        err32 = s.rel_error(y32, data["y"])
        q = torch.tensor([0.5, 0.9], device=err.device)
        e, e32 = torch.quantile(err.float(), q), torch.quantile(err32.float(), q)
        flops = 6.0 * 3 * n_train * epochs * sum(i * o for i, o in s.net.dims)
        rows.append({"hidden_layers": depth, "width": sg.HID, "epochs": epochs,
                     "train_states": n_train, "train_s": t_fit, "train_flops": flops,
                     "final_value_mse": hist[-1]["value_mse"],
                     "err_median": float(e[0]), "err_p90": float(e[1]),
                     "frac_err_below": {str(t): float((err <= t).float().mean()) for t in tols},
                     "fp32_err_median": float(e32[0]), "fp32_err_p90": float(e32[1]),
                     "fp32_frac_err_below": {str(t): float((err32 <= t).float().mean())
                                             for t in tols}})
        if log:
            log(rows[-1])
        del s, data
        torch.cuda.empty_cache()
    return {"surrogate_study": rows, "eval_states": n_eval,
            "error_metric": "per state ||(y_hat - y)/rms|| / ||y/rms|| over dT/dt and the 52 "
                            "molar rates", "train_flops": "6 x 3 passes (value, +-delta "
                            "directional) x states x epochs x sum of fan_in x fan_out"}


def lu_flops_per_state(nn):
    """FP64 flops of one Newton-matrix factorisation: forming I - g J (one FMA
    per entry), scaling the columns (one multiply per subdiagonal entry) and
    the rank-1 updates (one FMA per trailing entry and pivot)."""
    m = np.arange(1, nn)
    return 2 * nn * nn + int(m.sum()) + 2 * int((m * m).sum())


def implicit_bench(mech, ev, dev, n, order, steps, warmup, fp64_peak):
    """Implicit-step consumer of the Jacobian on n device-resident states:
    the Newton-matrix factorisation (pjg_lu_factor, dense Jacobian in, factors
    to a separate array), one solve (pjg_lu_solve) and a whole ROS2 step
    (pjg_ros2_step: 2 rates, 1 Jacobian, 1 factorisation, 2 solves).  Each
    timed alone with CUDA events over `steps` repetitions after `warmup`."""
    import torch
    integ = pkg("integrate")
    lib = pkg("_lib")
    nn = mech.nn
    P, phi = pkg("states").draw_states(mech.n_species, n, seed=2024, x_floor=1e-12)
    tP = torch.from_numpy(P).to(dev)
    tphi = torch.from_numpy(np.ascontiguousarray(phi.T) if order == "F" else phi).to(dev)
    h = torch.from_numpy(10.0 ** np.random.default_rng(5).uniform(-9, -6, n)).to(dev)
    jac = ev.jacobian(tP, tphi, order=order)
    lu = torch.empty_like(jac)
    b = torch.randn(tphi.shape, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)

    def timed(fn):
        for _ in range(max(3, warmup)):
            fn()
        torch.cuda.synchronize()
        l0 = lib.launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps, (lib.launch_count() - l0) / steps

    piv = [None]

    def factor():
        piv[0] = integ.lu_factor(jac, h, s=integ.ROS2_GAMMA, order=order, out=lu)[1]

    f_ms, f_launch = timed(factor)
    s_ms, s_launch = timed(lambda: integ.lu_solve(lu, piv[0], b, order=order))
    fs_ms, _ = timed(lambda: integ.lu_factor_sparse(ev, jac, h, s=integ.ROS2_GAMMA, order=order,
                                                    out=lu))
    ss_ms, _ = timed(lambda: integ.lu_solve_sparse(ev, lu, b, order=order))
    del jac, lu
    torch.cuda.empty_cache()
    y = torch.empty_like(tphi)
    err = torch.empty_like(tphi)
    st = integ.Ros2Stepper(ev, n, order=order)
    r_ms, r_launch = timed(lambda: st.step(tP, tphi, h, out=y, err=err))
    del st
    torch.cuda.empty_cache()
    st = integ.Ros2Stepper(ev, n, order=order, lu_kind="sparse")
    rs_ms, _ = timed(lambda: st.step(tP, tphi, h, out=y, err=err))
    fl = lu_flops_per_state(nn)
    f_rate = n / (f_ms * 1e-3)
    _, nnz_lu, fma_sp = integ.lu_plan_info(ev)
    # forming the entries and the updates; the column scalings (about 2 % more) are not counted
    fl_sp = 2 * nn * nn + 2 * fma_sp
    fs_rate = n / (fs_ms * 1e-3)
    lu_bytes = 8 * nn * nn
    res = {"states": n, "order": order, "h": "per state, log-uniform 1e-9 .. 1e-6 s",
           "factor": {"kernel": "lu_factor_kernel (one block of 2 warps per state, matrix in shared memory)",
                      "ms": f_ms, "states_per_s": f_rate, "launches": f_launch,
                      "flops_per_state": fl, "fp64_tflops": fl * f_rate / 1e12,
                      "fp64_frac": fl * f_rate / 1e12 / fp64_peak,
                      "fp64_peak_source": "measured DFMA probe (pjg_fp64_peak)",
                      "hbm_gbs": 2 * lu_bytes * f_rate / 1e9},
           "solve": {"kernel": "lu_solve_kernel (one thread per state)", "ms": s_ms,
                     "states_per_s": n / (s_ms * 1e-3), "launches": s_launch,
                     "alg_bytes_per_state": lu_bytes + 4 * nn + 16 * nn,
                     "hbm_gbs": (lu_bytes + 20 * nn) * n / (s_ms * 1e-3) / 1e9},
           "factor_sparse": {"kernel": "lu_sparse_kernel (static Markowitz order, no "
                                       "interchanges, filled pattern only)",
                             "ms": fs_ms, "states_per_s": fs_rate, "fma_per_state": fma_sp,
                             "nnz_lu": nnz_lu, "flops_per_state": fl_sp,
                             "fp64_tflops": fl_sp * fs_rate / 1e12,
                             "fp64_frac": fl_sp * fs_rate / 1e12 / fp64_peak},
           "solve_sparse": {"kernel": "lu_sparse_solve_kernel", "ms": ss_ms,
                            "states_per_s": n / (ss_ms * 1e-3)},
           "ros2_step": {"ms": r_ms, "states_per_s": n / (r_ms * 1e-3), "launches": r_launch,
                         "path": "Ros2Stepper.step -> pjg_ros2_step (partial pivoting)"},
           "ros2_step_sparse": {"ms": rs_ms, "states_per_s": n / (rs_ms * 1e-3),
                                "path": "Ros2Stepper(lu_kind='sparse').step -> pjg_ros2_step"}}
    del st, y, err
    torch.cuda.empty_cache()
    return res


def implicit_large_bench(dev, n, fp64_peak, steps=2, warmup=1):
    """The Newton-matrix factorisation beyond shared memory: the seeded
    500-species synthetic mechanism (NN = 501), n states in C order, the dense
    Jacobian factored by the blocked global-memory kernel, one solve, and one
    whole ROS2 step (partial pivoting).  The oracle's operation count per
    state (2/3 NN^3 + ...) sets the FP64 fraction."""
    import torch
    integ = pkg("integrate")
    mech = load_mech("synthetic500")
    ev = pkg("api").Evaluator(mech)
    nn = mech.nn
    P, phi = pkg("states").draw_states(mech.n_species, n, seed=2025, x_floor=1e-12)
    tP = torch.from_numpy(P).to(dev)
    tphi = torch.from_numpy(phi).to(dev)
    h = torch.from_numpy(10.0 ** np.random.default_rng(6).uniform(-12, -9, n)).to(dev)
    jac = ev.jacobian(tP, tphi, order="C")
    lu = torch.empty_like(jac)
    b = torch.randn(tphi.shape, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)

    def timed(fn):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    piv = [None, None]

    def factor():
        _, piv[0], piv[1] = integ.lu_factor(jac, h, s=integ.ROS2_GAMMA, order="C", out=lu)

    f_ms = timed(factor)
    s_ms = timed(lambda: integ.lu_solve(lu, piv[0], b, order="C"))
    singular = int((piv[1] != 0).sum())
    del jac, lu
    torch.cuda.empty_cache()
    y, err = torch.empty_like(tphi), torch.empty_like(tphi)
    st = integ.Ros2Stepper(ev, n, order="C")
    r_ms = timed(lambda: st.step(tP, tphi, h, out=y, err=err))
    fl = lu_flops_per_state(nn)
    f_rate = n / (f_ms * 1e-3)
    res = {"mechanism": "synthetic-500 (500 species, 2,500 reactions), NN = %d" % nn,
           "states": n, "order": "C", "h": "per state, log-uniform 1e-12 .. 1e-9 s",
           "factor": {"kernel": "lu_factor_big_kernel (one block per state, panels of 16 columns "
                                "in shared memory, the matrix in global memory)",
                      "ms": f_ms, "states_per_s": f_rate, "flops_per_state": fl,
                      "fp64_tflops": fl * f_rate / 1e12, "fp64_frac": fl * f_rate / 1e12 / fp64_peak,
                      "fp64_peak_source": "measured DFMA probe (pjg_fp64_peak)",
                      "states_with_zero_pivot": singular,
                      "zero_pivot_note": "the seeded synthetic mechanism's Jacobians reach 1e166; at "
                                         "these steps elimination leaves exactly zero pivots, as in "
                                         "the oracle (LAPACK's order); the work per state is the same"},
           "solve": {"kernel": "lu_solve_big_kernel (one block per state, vector in shared memory, "
                               "column sweeps)",
                     "ms": s_ms, "states_per_s": n / (s_ms * 1e-3),
                     "hbm_gbs": (8 * nn * nn + 20 * nn) * n / (s_ms * 1e-3) / 1e9},
           "ros2_step": {"ms": r_ms, "states_per_s": n / (r_ms * 1e-3),
                         "path": "Ros2Stepper.step -> pjg_ros2_step (partial pivoting)"}}
    del st, y, err
    torch.cuda.empty_cache()
    return res


# ------------------------------------------------------------------ the line

def headline_config(args, mech):
    """The `config` object of the headline line (shared by both arms)."""
    label = MECHS[args.mech][0]
    n = args.states
    n_out, n_in = io_sizes(mech, args.kernel, args.format)
    if args.kernel == "jacobian":
        what = ("%s %s FP64 %sJacobian, %s order, %d states"
                % (label, "dense" if args.format == "full" else
                   ("sparse CCS" if args.order == "F" else "sparse CRS"),
                   "approximate " if args.jac_type == "approximate" else "", args.order, n))
    else:
        what = ("%s FP64 %s, %s order, %d states"
                % (label, "species rates" if args.kernel == "rates" else "J^T v", args.order, n))
    return {"workload": what, "mechanism": MECHS[args.mech][2], "states": n, "order": args.order,
            "jac_format": args.format, "jac_type": args.jac_type, "conp": True,
            "l2": "inputs %.0f MB and outputs %.0f MB, both larger than L2 (126 MB): no flush"
                  % (8e-6 * n_in * n, 8e-6 * n_out * n)}


def headline_metric(args):
    metric, unit, _ = KERNELS[args.kernel]
    return metric.replace("GRI-30", MECHS[args.mech][0]), unit


def run_reference(args):
    """The reference arm: the reference's CPU implementation of the headline
    on this host's cores, each step a bounded sample of the workload."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    mech = load_mech(args.mech, args.jac_type)
    metric, unit = headline_metric(args)
    n = args.cpu_sample
    cb, sec = cpu_reference_run(mech, n, args.steps, warmup=args.warmup, mech_name=args.mech,
                                kernel=args.kernel)
    out = {"metric": metric, "value": cb["value"], "unit": unit, "impl": "reference",
           "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": headline_config(args, mech),
           "cpu_baseline": cb,
           "e2e": {"value": cb["value"], "unit": unit, "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return 0


def run_gpu(args):
    """One rank of the GPU arm (rank and world from the environment)."""
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    sh = pkg("shard")
    if world > 1:
        sh.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = pkg("_lib")
    api = pkg("api")
    states = pkg("states")
    mech = load_mech(args.mech, args.jac_type)
    ev = api.Evaluator(mech)
    n = args.states
    nn = mech.nn
    metric, unit = headline_metric(args)
    kname = KERNELS[args.kernel][2]
    n_out, n_in = io_sizes(mech, args.kernel, args.format)
    P, phi = states.draw_states(mech.n_species, n, seed=1000 + rank, x_floor=1e-12)
    x = np.ascontiguousarray(phi.T) if args.order == "F" else phi
    tP = torch.from_numpy(P).to(dev)
    tphi = torch.from_numpy(x).to(dev)
    out = torch.empty(n * n_out, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    tv = None
    if args.kernel == "vjp":
        tv = torch.from_numpy(np.random.default_rng(77).standard_normal(x.shape)).to(dev)

    def step():
        if args.kernel == "jacobian":
            ev.jacobian(tP, tphi, order=args.order, conp=True, jac_format=args.format, out=out)
        elif args.kernel == "rates":
            ev.species_rates(tP, tphi, order=args.order, conp=True, out=out.view(tphi.shape))
        else:
            ev.vjp(tP, tphi, tv, order=args.order, conp=True, out=out.view(tphi.shape))

    for _ in range(max(3, args.warmup)):
        step()
    torch.cuda.synchronize()
    fp64_peak = ctypes.c_double()
    lib.check("pjg_fp64_peak", lib.load().pjg_fp64_peak(ctypes.byref(fp64_peak)))
    fp64_peak = fp64_peak.value
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    sh.barrier()
    torch.cuda.synchronize()
    launches0 = lib.launch_count()
    lib.profile_begin()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    n_eval, eval_ms = lib.profile_end()
    launches = lib.launch_count() - launches0
    sh.barrier()
    ms = sh.max_over_ranks(e0.elapsed_time(e1), device=dev)  # the slowest rank
    clk = clocks.stop()
    ms_step = ms / args.steps
    value = world * n * args.steps / (ms * 1e-3)

    # roofline of the timed evaluation kernel
    bpsi = alg_bytes_per_state(nn, n_out, n_in)
    per_launch = n / max(1, n_eval // args.steps)  # states one launch covers
    achieved = bpsi * n * args.steps / (eval_ms * 1e-3) / 1e9
    peak, peak_src = hbm_peak()
    krate = n * args.steps / (eval_ms * 1e-3)  # states/s of the evaluation kernel alone
    fp64 = fp64_roofline(args.mech, args.kernel, args.format, args.order, krate, fp64_peak)
    key = "%s_%s_%s" % (args.kernel, args.format if args.kernel == "jacobian" else "na", args.order)
    if args.mech != "gri30":
        key = args.mech + "_" + key
    nc = read_json(NCU_COUNTS).get(key, {})
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak,
                "traffic": (nc["dram_bytes_per_state"] * per_launch
                            if nc.get("dram_bytes_per_state") else None),
                "peak_source": peak_src, "kernel": kname, "alg_bytes_per_state": bpsi,
                "eval_ms_per_step": eval_ms / args.steps, "eval_launches": n_eval,
                "binding": "fp64 pipe: see fp64.frac (algorithmic flops) and fp64.pipe_frac "
                           "(executed FP64 instructions x rate / DFMA rate)",
                "fp64": fp64}

    # parity of the timed output itself (rank 0; every rank runs the same code)
    parity = None
    if rank == 0 and not args.no_parity:
        chunk = lib.eval_chunk(ev.handle, KIND[args.kernel], n, args.order,
                               0 if args.format == "full" else 1)
        parity = parity_check(mech, ev, args.kernel, args.format, args.order, P, phi, out, tP,
                              tphi, tv, chunk=chunk)

    # the device-timed leg is done: its output goes back to the pool, so the
    # kernel object below sizes its chunks against what the device really has
    del out
    torch.cuda.empty_cache()

    # end to end through the reference-facing kernel object, host buffers
    # (page-locked in place); with several ranks each takes n / world states,
    # so the host holds one problem's arrays in all
    e2e = None
    if not args.no_e2e and args.kernel != "vjp":
        a, b = sh.state_range(n, rank, world) if world > 1 else (0, n)
        ne = b - a
        xe = np.ascontiguousarray(phi[a:b].T) if args.order == "F" else phi[a:b]
        mod = api.pywrap(mech, order=args.order, conp=True, jac_format=args.format)
        kobj = (mod.PyJacobianKernel if args.kernel == "jacobian" else mod.PySpecies_RatesKernel)(ne, 1)
        hm = pkg("hostmem")
        hP = hm.empty((ne,))
        hP[:] = P[a:b]
        hphi = hm.empty(xe.shape)
        hphi[:] = xe
        hout = hm.empty((ne * n_out,))
        for _ in range(2):  # warm-up calls
            kobj(hP, hphi, hout)
        k2 = max(1, min(args.steps, 5))
        sh.barrier()
        calls = []
        for _ in range(k2):
            t0 = time.perf_counter()
            kobj(hP, hphi, hout)
            calls.append(time.perf_counter() - t0)
        sec = sh.max_over_ranks(sum(calls) / k2)
        e2e = {"value": world * ne / sec, "unit": unit,
               "h2d_bytes_per_step": int(hP.nbytes + hphi.nbytes) * world,
               "d2h_bytes_per_step": int(hout.nbytes) * world, "steps": k2,
               "states_per_rank": ne,
               "call_ms": [round(c * 1e3, 1) for c in calls],
               "median_call_ms": round(float(np.median(calls)) * 1e3, 1),
               "path": "%s(problem_size, work_size)(param, phi, out), host arrays page-locked "
                       "in place (hostmem.empty)" % type(kobj).__name__}
        e2e.update(hm.placement_info(hout))
        kobj.close()
        # the host link alone: the same bytes device -> these host arrays,
        # copied from one device buffer in 4 GiB pieces (untimed by the line)
        import torch
        dbuf = torch.empty(min(hout.size, 1 << 29), dtype=torch.float64, device=dev)
        hv = torch.from_numpy(hout)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for o in range(0, hout.size, dbuf.numel()):
            m = min(dbuf.numel(), hout.size - o)
            hv[o:o + m].copy_(dbuf[:m], non_blocking=True)
        torch.cuda.synchronize()
        t_link = time.perf_counter() - t0
        del dbuf, hv
        e2e["link"] = {"d2h_gbs": hout.nbytes / t_link / 1e9,
                       "d2h_floor_ms_per_step": t_link * 1e3,
                       "fastest_call_over_floor": min(calls) / t_link,
                       "what": "the step's output bytes copied device -> the same page-locked "
                               "host array alone, in 4 GiB pieces: the host link's floor"}
        del hout, hphi, hP

    single = world == 1 and rank == 0
    cpu = None
    cpu_cache = {}
    if rank == 0 and not args.no_cpu:
        cpu, _ = cpu_reference_run(mech, args.cpu_sample, 1, mech_name=args.mech,
                                   kernel=args.kernel)
        cpu_cache[(args.mech, args.kernel)] = cpu

    implicit = None
    if single and not args.no_implicit and args.kernel == "jacobian" and nn <= 169:
        implicit = implicit_bench(mech, ev, dev, n, args.order, args.steps, args.warmup, fp64_peak)
        if args.mech == "gri30" and args.format == "full" and args.jac_type == "exact" and \
                args.implicit_large_states > 0:
            implicit["synthetic500"] = implicit_large_bench(dev, args.implicit_large_states, fp64_peak)

    configs = None
    if single and not args.no_configs and args.mech == "gri30" and args.kernel == "jacobian" \
            and args.format == "full" and args.order == "F" and args.jac_type == "exact":
        configs = {}
        torch.cuda.empty_cache()
        for key_, mn, kern, fmt, order, nst, cs in CONFIGS:
            configs[key_] = measure_config(key_, mn, kern, fmt, order, nst, cs, dev,
                                           min(args.steps, 10), args.warmup, fp64_peak, cpu_cache)
            print(json.dumps({key_: {k: configs[key_][k] for k in ("value", "unit")}}),
                  file=sys.stderr)

    sur = None
    if single and not args.no_surrogate and args.kernel == "jacobian" and args.mech == "gri30":
        torch.cuda.empty_cache()
        sur = surrogate_bench(mech, ev, dev, args.sur_train, args.sur_epochs, args.sur_eval,
                              log=lambda h: print(json.dumps(h), file=sys.stderr))

    if rank == 0:
        line = {"metric": metric, "value": value, "unit": unit, "n_gpus": world,
                "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms_step,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic",
                "config": headline_config(args, mech),
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": launches, "clocks": clk, "parity": parity,
                "configs": configs, "surrogate": sur, "implicit_step": implicit}
        print(json.dumps(line))
    sh.barrier()
    sh.destroy_process_group()
    return 0


def parse_args(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--states", type=int, default=1 << 20)
    ap.add_argument("--format", default="full", choices=["full", "sparse"])
    ap.add_argument("--order", default="F", choices=["C", "F"])
    ap.add_argument("--cpu-sample", type=int, default=None,
                    help="states per CPU-baseline step (default: a few seconds of work on 16 cores "
                         "for the reference's code; 2,048 for the 500-species oracle port)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-parity", action="store_true", help="skip the headline's sampled parity")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the other benchmark configurations")
    ap.add_argument("--no-surrogate", action="store_true")
    ap.add_argument("--no-implicit", action="store_true",
                    help="skip the implicit-step block (Newton-matrix LU, solve, ROS2 step)")
    ap.add_argument("--implicit-large-states", type=int, default=4096,
                    help="states of the synthetic-500 Newton-matrix block (0: skip it)")
    ap.add_argument("--sur-train", type=int, default=1 << 22)
    ap.add_argument("--sur-epochs", type=int, default=60)
    ap.add_argument("--sur-eval", type=int, default=1 << 22)
    ap.add_argument("--surrogate-study", action="store_true",
                    help="only the surrogate's capacity study (depth x epochs x training states); "
                         "prints one JSON line")
    ap.add_argument("--jac-type", default="exact", choices=["exact", "approximate"],
                    help="Jacobian type: exact (headline) or the reference's approximate type, "
                         "without the bath-gas terms")
    ap.add_argument("--mech", default="gri30", choices=sorted(MECHS),
                    help="mechanism: GRI-Mech 3.0 (headline), H2/O2, or the 500-species synthetic")
    ap.add_argument("--kernel", default="jacobian", choices=sorted(KERNELS),
                    help="evaluation timed: the Jacobian (headline), species rates or J^T v")
    args = ap.parse_args(argv)
    if args.cpu_sample is None:
        args.cpu_sample = {"gri30": 131072, "h2o2": 1048576, "synthetic500": 2048}[args.mech]
    return args


def main(argv=None):
    args = parse_args(argv)
    if args.impl == "reference":
        return run_reference(args)
    if args.surrogate_study:
        import torch
        dev = torch.device("cuda:0")
        mech = load_mech("gri30")
        res = surrogate_study(mech, pkg("api").Evaluator(mech), dev,
                              log=lambda r: print(json.dumps(r), file=sys.stderr, flush=True))
        print(json.dumps(res))
        return 0
    sh = pkg("shard")
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # not started by torchrun: one process per GPU, spawned here
        return sh.spawn(_rank_main, args.gpus, (args,))
    return run_gpu(args)


def _rank_main(args):
    return run_gpu(args)


if __name__ == "__main__":
    sys.exit(main())

"""Benchmark: GRI-Mech 3.0 dense FP64 analytical Jacobians on one GB300.

Workload (the headline configuration): GRI-Mech 3.0 (53 species, 325
reactions), 1,048,576 seeded synthetic states (T ~ U(800, 2200) K,
P log-uniform 1-25 atm, X ~ Dirichlet(0.5) floored at 1e-12, V = 1 m^3),
constant pressure, F data order, dense 54 x 54 Jacobian.  One step = one
Jacobian evaluation of all states (pjg_jacobian).  Inputs (453 MB) and outputs
(24.5 GB) are larger than L2, so no flush is needed between steps.

Other configurations: ``--mech h2o2`` (H2/O2), ``--mech synthetic500`` (the
seeded 500-species, 2,500-reaction mechanism), ``--format sparse``,
``--order C``, ``--kernel rates|vjp``, ``--states N``.

Prints one JSON line (rank 0).  ``--impl reference`` times the reference's CPU
implementation of the same path on the host cores instead: the shim-compiled
shipped GRI or H2/O2 kernels in oracle/_ref when they load here, else the C
oracle (the CPU restatement of the reference) with OpenMP on all cores.
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
# measured FP64 instruction / DRAM counts per state (ncu), see profiles/
COUNTS = os.path.join(ROOT, "profiles", "gri30_kernel_counts.json")


def alg_bytes_per_state(nn, n_out, n_in=None):
    """Algorithmic HBM bytes per state: read phi (NN) + param (+ v for J^T v),
    write n_out values."""
    return 8 * (nn + 1 if n_in is None else n_in) + 8 * n_out


def pkg(sub=None):
    return importlib.import_module(PKG + ("." + sub if sub else ""))


def load_gri(jac_type="exact"):
    return pkg().load_mechanism(os.path.join(ROOT, "data", "grimech30.inp"),
                                os.path.join(ROOT, "data", "thermo30.dat"), jac_type=jac_type)


# --mech: the benchmark configurations' mechanisms, their label and the
# reference's shipped kernels for the CPU baseline (None: the C oracle port)
MECHS = {
    "gri30": ("GRI-30", "ch4", "grimech30 (53 species, 325 reactions)"),
    "h2o2": ("H2/O2", "h2o2", "h2o2 (9 species, 28 reactions)"),
    "synthetic500": ("synthetic-500", None, "seeded synthetic (500 species, 2,500 reactions)"),
}


def load_mech(name, jac_type="exact"):
    if name == "gri30":
        return load_gri(jac_type)
    if name == "h2o2":
        return pkg().load_mechanism(os.path.join(ROOT, "data", "h2o2.inp"), jac_type=jac_type)
    import tempfile
    path = os.path.join(tempfile.gettempdir(), "pyjac_gb300_synthetic500_seed0.inp")
    if not os.path.exists(path):
        pkg("mech.synthetic").write(path + ".tmp")  # defaults: 500 species, 2,500 reactions
        os.replace(path + ".tmp", path)
    return pkg().load_mechanism(path, jac_type=jac_type)


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


def cpu_reference_run(mech, n_sample, steps, seed=1, warmup=1, mech_name="gri30"):
    """Time the reference's CPU implementation: states/s and a description."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    orc = importlib.import_module("oracle")
    states = pkg("states")
    P, phi = states.draw_states(mech.n_species, n_sample, seed=seed, x_floor=1e-12)
    threads = cpu_threads()
    kind, fn = None, None
    label, shipped, _ = MECHS[mech_name]
    if shipped and orc.RefKernels.available(shipped):
        try:
            ref = orc.RefKernels(shipped)
            phiF = np.ascontiguousarray(phi.T)
            kind = "reference"
            desc = ("reference shipped %s kernels (examples/opencl/%s, %s), shim-compiled"
                    % (label, shipped, "sparse CCS" if shipped == "ch4" else "dense"))

            def fn():
                ref.jacobian_F(P, phiF, nthreads=threads)
        except OSError:
            kind = None
    if kind is None:
        o = orc.Oracle(mech)
        kind = "port"
        desc = "C oracle (CPU restatement of the reference), dense Jacobian, OpenMP"

        def fn():
            o.jacobian(P, phi, conp=True, nthreads=threads)
    for _ in range(max(1, warmup)):  # untimed calls first (the reference's main times its second)
        fn()
    ts = []
    for _ in range(max(1, steps)):
        t0 = time.perf_counter()
        fn()
        ts.append(time.perf_counter() - t0)
    sec = float(np.mean(ts))
    return {"value": n_sample / sec, "unit": UNIT, "cores": threads, "kind": kind,
            "sample": "%d %s states per step, %s" % (n_sample, label, desc)}, sec


def surrogate_bench(mech, ev, dev, n_train, epochs, n_eval, log=None):
    """Train the BF16 surrogate on n_train states (Sobolev loss), then report its
    error against the FP64 kernel and the wdot speedup at several tolerances on
    n_eval fresh states (FP64 fallback included in the timed path)."""
    import torch
    sg = pkg("surrogate")
    s = sg.Surrogate(mech, device=dev, evaluator=ev)
    t0 = time.time()
    hist = s.fit(n_train=n_train, epochs=epochs, batch=16384, lr=2e-3, log=log)
    torch.cuda.synchronize()
    t_train = time.time() - t0
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
    t_net, raw = timed(lambda: s.predict(P, phi))
    y_hat = torch.cat([raw[0][:, :1], raw[0][:, 2:]], dim=1)
    err = s.rel_error(y_hat, data["y"])
    q = torch.quantile(err[: min(len(err), 1 << 24)].float(), torch.tensor([0.5, 0.9, 0.99], device=dev))
    qmax = torch.quantile(s.max_rel_error(y_hat, data["y"]).float(),
                          torch.tensor([0.5, 0.9, 0.99], device=dev))
    tols = []
    for tol in (1e-1, 1e-2, 1e-3):
        t_tol, (out, info) = timed(lambda: s.species_rates(P, phi, tol=tol, return_info=True), reps=1)
        yo = torch.cat([out[:, :1], out[:, 2:]], dim=1)
        e2 = s.rel_error(yo, data["y"])
        tols.append({"tol": tol, "ms": t_tol, "fallback_frac": info["fallback_frac"],
                     "speedup_vs_fp64": t_fp64 / t_tol,
                     "frac_states_within_tol": float((e2 <= tol).float().mean()),
                     "p99_err": float(torch.quantile(e2.float(), 0.99))})
    return {"network": "54 -> 4x256 SiLU -> 53 (+1 error estimate), BF16 weights/activations, "
                       "FP32 accumulate, tcgen05 GEMMs",
            "train_states": n_train, "epochs": epochs, "train_s": t_train,
            "final_value_mse": hist[-1]["value_mse"], "final_sobolev_mse": hist[-1]["sobolev_mse"],
            "eval_states": n_eval, "fp64_rates_ms": t_fp64, "network_ms": t_net,
            "network_speedup_vs_fp64": t_fp64 / t_net,
            "err_median": float(q[0]), "err_p90": float(q[1]), "err_p99": float(q[2]),
            "worst_component_err_median": float(qmax[0]), "worst_component_err_p90": float(qmax[1]),
            "frac_err_below": {"1e-1": float((err <= 1e-1).float().mean()),
                               "1e-2": float((err <= 1e-2).float().mean()),
                               "1e-3": float((err <= 1e-3).float().mean())},
            "with_fallback": tols,
            "error_metric": "per state ||(y_hat - y)/rms|| / ||y/rms|| over dT/dt and the 52 molar "
                            "rates (rms over training states); worst component: "
                            "max_k |y_hat - y| / (|y| + 1e-3 rms_k)"}


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


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    mech = load_mech(args.mech)
    n = args.cpu_sample
    cb, sec = cpu_reference_run(mech, n, args.steps, warmup=args.warmup, mech_name=args.mech)
    out = {"metric": METRIC.replace("GRI-30", MECHS[args.mech][0]), "value": cb["value"],
           "unit": UNIT, "impl": "reference",
           "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": sec * 1e3, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": "%s FP64 Jacobian, %d states per step on host cores"
                                  % (MECHS[args.mech][0], n),
                      "mechanism": MECHS[args.mech][2], "states": n, "conp": True},
           "cpu_baseline": cb,
           "e2e": {"value": cb["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                   "d2h_bytes_per_step": 0}}
    print(json.dumps(out))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--states", type=int, default=1 << 20)
    ap.add_argument("--format", default="full", choices=["full", "sparse"])
    ap.add_argument("--order", default="F", choices=["C", "F"])
    ap.add_argument("--cpu-sample", type=int, default=None,
                    help="states per CPU-baseline step (default: about 10 s of work on 16 cores "
                         "for the reference's code; 2,048 for the 500-species oracle port)")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-surrogate", action="store_true")
    ap.add_argument("--no-implicit", action="store_true",
                    help="skip the implicit-step block (Newton-matrix LU, solve, ROS2 step)")
    ap.add_argument("--sur-train", type=int, default=1 << 22)
    ap.add_argument("--sur-epochs", type=int, default=12)
    ap.add_argument("--sur-eval", type=int, default=1 << 22)
    ap.add_argument("--jac-type", default="exact", choices=["exact", "approximate"],
                    help="Jacobian type: exact (headline) or the reference's approximate type, "
                         "without the bath-gas terms")
    ap.add_argument("--mech", default="gri30", choices=sorted(MECHS),
                    help="mechanism: GRI-Mech 3.0 (headline), H2/O2, or the 500-species synthetic")
    ap.add_argument("--kernel", default="jacobian", choices=sorted(KERNELS),
                    help="evaluation timed: the Jacobian (headline), species rates or J^T v")
    args = ap.parse_args()
    if args.cpu_sample is None:
        args.cpu_sample = {"gri30": 524288, "h2o2": 2097152, "synthetic500": 2048}[args.mech]
    if args.impl == "reference":
        return run_reference(args)

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    lib = pkg("_lib")
    api = pkg("api")
    states = pkg("states")
    mech = load_mech(args.mech, args.jac_type)
    ev = api.Evaluator(mech)
    n = args.states
    nn = mech.nn
    metric, unit, kname = KERNELS[args.kernel]
    label = MECHS[args.mech][0]
    metric = metric.replace("GRI-30", label)
    if args.kernel == "jacobian":
        n_out = nn * nn if args.format == "full" else mech.jac_nnz()
        n_in = nn + 1
    else:
        n_out = nn
        n_in = nn + 1 if args.kernel == "rates" else 2 * nn + 1
    P, phi = states.draw_states(mech.n_species, n, seed=1000 + rank, x_floor=1e-12)
    x = np.ascontiguousarray(phi.T) if args.order == "F" else phi
    tP = torch.from_numpy(P).to(dev)
    tphi = torch.from_numpy(x).to(dev)
    out = torch.empty(n * n_out, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
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
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
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
    ms = e0.elapsed_time(e1)
    ms = pkg("shard").max_over_ranks(ms, device=dev)  # the slowest rank
    clk = clocks.stop()
    ms_step = ms / args.steps
    value = world * n * args.steps / (ms * 1e-3)

    # roofline of the timed evaluation kernel
    bpsi = alg_bytes_per_state(nn, n_out, n_in)
    per_launch = n / max(1, n_eval // args.steps)  # states one launch covers
    achieved = bpsi * n * args.steps / (eval_ms * 1e-3) / 1e9
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    hbm_peak, peak_src = 6800.0, "fallback"
    if os.path.exists(peaks_path):
        with open(peaks_path) as fh:
            hbm_peak = float(json.load(fh).get("hbm_gbs", hbm_peak))
        peak_src = "measured"
    key = "%s_%s_%s" % (args.kernel, args.format if args.kernel == "jacobian" else "na", args.order)
    if args.mech != "gri30":
        key = args.mech + "_" + key
    counts = {}
    if os.path.exists(COUNTS):
        with open(COUNTS) as fh:
            counts = json.load(fh).get(key, {})
    krate = n * args.steps / (eval_ms * 1e-3)  # states/s of the evaluation kernel alone
    fp64 = {"peak": fp64_peak.value, "unit": "TFLOP/s",
            "peak_source": "measured DFMA probe (pjg_fp64_peak)"}
    if counts:
        fl, ins = counts["fp64_flops_per_state"], counts["fp64_inst_per_state"]
        fp64.update({"achieved": fl * krate / 1e12, "frac": fl * krate / 1e12 / fp64_peak.value,
                     "flops_per_state": fl, "pipe_inst_per_state": ins,
                     "pipe_frac": ins * krate / (fp64_peak.value * 1e12 / 2),
                     "counts": "ncu, %s (profiles/)" % counts.get("case", "")})
    roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                "frac": achieved / hbm_peak,
                "traffic": (counts["dram_bytes_per_state"] * per_launch
                            if counts.get("dram_bytes_per_state") else None),
                "peak_source": peak_src, "kernel": kname, "alg_bytes_per_state": bpsi,
                "eval_ms_per_step": eval_ms / args.steps, "eval_launches": n_eval,
                "binding": "fp64 pipe: see fp64.pipe_frac (FP64 instructions x rate / DFMA rate)",
                "fp64": fp64}

    # the device-timed leg is done: its output goes back to the pool, so the
    # kernel object below sizes its chunks against what the device really has
    del out
    torch.cuda.empty_cache()

    # end to end through the reference-facing kernel object, host buffers (pinned)
    e2e = None
    if not args.no_e2e and args.kernel != "vjp":
        mod = api.pywrap(mech, order=args.order, conp=True, jac_format=args.format)
        kobj = (mod.PyJacobianKernel if args.kernel == "jacobian" else mod.PySpecies_RatesKernel)(n, 1)
        # host arrays page-locked in place (pjg_host_register): steadier than
        # cudaHostAlloc buffers once other processes have churned host memory
        hm = pkg("hostmem")
        hP = hm.empty(P.shape)
        hP[:] = P
        hphi = hm.empty(x.shape)
        hphi[:] = x
        hout = hm.empty((n * n_out,))
        for _ in range(2):  # warm-up calls
            kobj(hP, hphi, hout)
        k2 = max(1, min(args.steps, 5))
        if world > 1:
            torch.distributed.barrier()
        calls = []
        for _ in range(k2):
            t0 = time.perf_counter()
            kobj(hP, hphi, hout)
            calls.append(time.perf_counter() - t0)
        sec = sum(calls) / k2
        e2e = {"value": world * n / sec, "unit": unit,
               "h2d_bytes_per_step": int(hP.nbytes + hphi.nbytes),
               "d2h_bytes_per_step": int(hout.nbytes), "steps": k2,
               "call_ms": [round(c * 1e3, 1) for c in calls],
               "median_call_ms": round(float(np.median(calls)) * 1e3, 1),
               "path": "%s(problem_size, work_size)(param, phi, out), host arrays page-locked "
                       "in place (hostmem.empty)" % type(kobj).__name__}
        kobj.close()
        del hout

    cpu = None
    if rank == 0 and not args.no_cpu and args.kernel == "jacobian":
        cpu, _ = cpu_reference_run(mech, args.cpu_sample, 1, mech_name=args.mech)

    implicit = None
    if not args.no_implicit and args.kernel == "jacobian" and nn <= 169:
        implicit = implicit_bench(mech, ev, dev, n, args.order, args.steps, args.warmup,
                                  fp64_peak.value)

    sur = None
    if not args.no_surrogate and args.kernel == "jacobian" and args.mech == "gri30":
        torch.cuda.empty_cache()
        sur = surrogate_bench(mech, ev, dev, args.sur_train, args.sur_epochs, args.sur_eval,
                              log=lambda h: print(json.dumps(h), file=sys.stderr))

    if rank == 0:
        line = {"metric": metric, "value": value, "unit": unit, "n_gpus": world,
                "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms_step,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic",
                "config": {"workload": ("%s %s FP64 %sJacobian, %s order, %d states"
                                        % (label, "dense" if args.format == "full" else
                                           ("sparse CCS" if args.order == "F" else "sparse CRS"),
                                           "approximate " if args.jac_type == "approximate" else "",
                                           args.order, n)) if args.kernel == "jacobian" else
                           ("%s FP64 %s, %s order, %d states"
                            % (label, "species rates" if args.kernel == "rates" else "J^T v",
                               args.order, n)),
                           "mechanism": MECHS[args.mech][2],
                           "states": n, "order": args.order, "jac_format": args.format,
                           "jac_type": args.jac_type,
                           "conp": True,
                           "l2": "inputs %.0f MB and outputs %.0f MB, both larger than L2 (126 MB): "
                                 "no flush" % (8e-6 * n_in * n, 8e-6 * n_out * n)},
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e,
                "gpu_launches": launches, "clocks": clk, "surrogate": sur,
                "implicit_step": implicit}
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

"""Write data/fp64_op_counts.json: FP64 operations per state of the
reference's formulation, counted by the oracle (flop_count.cpp).

Measurement infrastructure: the counts are the algorithmic FP64 work of
species rates and of the analytical Jacobian as pyjac/core/rate_subs.py and
pyjac/core/create_jacobian.py formulate them (the oracle restates those
formulas operation for operation), averaged over seeded states of the
benchmark distribution.  bench.py divides them by the measured kernel time
for the FP64 roofline; tests/test_oracle.py checks that this file matches a
fresh count.

    python oracle/count_flops.py
"""
import importlib
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
OUT = os.path.join(ROOT, "data", "fp64_op_counts.json")
# states averaged per mechanism (the synthetic mechanism's dense Jacobian is
# large; its counts vary little from state to state)
SAMPLE = {"h2o2": 256, "gri30": 256, "synthetic500": 8}
SEED = 3


def _mech(name):
    pj = importlib.import_module("pyjac-v2_gb300")
    if name == "gri30":
        return pj.load_mechanism(os.path.join(ROOT, "data", "grimech30.inp"),
                                 os.path.join(ROOT, "data", "thermo30.dat"))
    if name == "h2o2":
        return pj.load_mechanism(os.path.join(ROOT, "data", "h2o2.inp"))
    import tempfile
    path = os.path.join(tempfile.gettempdir(), "pyjac_gb300_synthetic500_seed0.inp")
    if not os.path.exists(path):
        importlib.import_module("pyjac-v2_gb300.mech.synthetic").write(path + ".tmp")
        os.replace(path + ".tmp", path)
    return pj.load_mechanism(path)


def count(name, n=None):
    """{'rates': {...}, 'jacobian': {...}, 'vjp': {...}} per-state counts of one mechanism."""
    for p in (ROOT, HERE):
        if p not in sys.path:
            sys.path.insert(0, p)
    orc = importlib.import_module("oracle")
    states = importlib.import_module("pyjac-v2_gb300.states")
    mech = _mech(name)
    n = n or SAMPLE[name]
    P, phi = states.draw_states(mech.n_species, n, seed=SEED, x_floor=1e-12)
    o = orc.Oracle(mech)
    out = {"states": n, "seed": SEED, "nn": mech.nn}
    for kind in ("rates", "jacobian"):
        out[kind] = {k: round(v, 3) for k, v in o.op_counts(P, phi, kind).items()}
    # J^T v has no reference counterpart: the reference's route to it is the
    # analytical Jacobian followed by a dense matrix-vector product
    vjp = dict(out["jacobian"])
    vjp["fma"] = vjp["fma"] + mech.nn * mech.nn
    vjp["flops"] = vjp["flops"] + 2 * mech.nn * mech.nn
    out["vjp"] = vjp
    return out


def main():
    res = {"what": "FP64 operations per state of the reference's formulation, counted by "
                   "oracle/flop_count.cpp; flops = add + mul + div + 2 fma; minmax and the "
                   "transcendental functions are counted separately (not in flops)",
           "mechanisms": {name: count(name) for name in SAMPLE}}
    with open(OUT, "w") as fh:
        json.dump(res, fh, indent=1, sort_keys=True)
        fh.write("\n")
    print("written", OUT)


if __name__ == "__main__":
    main()

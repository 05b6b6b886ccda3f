"""Generate the golden fixtures under tests/golden/ from the reference itself.

Run in a tree where the reference is available (--reference, else the
PYJAC_REFERENCE environment variable, else the default of oracle/build_ref.py):

    python tests/golden/make_golden.py [--reference DIR]

Writes
* ``tables_<mech>.npz``: the reference front end's tables and Jacobian index
  arrays (pyjac/core/mech_interpret.py read_mech -> create_jacobian.py
  find_last_species -> utils.py reassign_species_lists ->
  create_jacobian.py determine_jac_inds, hybrid rate specialisation), flattened
  to ``section/key`` arrays, for h2o2, gri30, testmech and synthetic_small;
* ``ref_<mech>.npz`` for h2o2 and gri30: seeded states and the outputs of the
  reference's shipped generated kernels (examples/opencl/{h2o2,ch4},
  shim-compiled by oracle/build_ref.py): dphi and the Jacobian in the shipped
  format (dense F for H2/O2, sparse CCS for GRI-30), F order, conp; and the
  shipped chem_utils outputs (cp, h, b) over a temperature sweep through both
  NASA ranges and beyond the 100 K / 10,000 K guards;
* ``jacapprox_<mech>.npz``: the reference front end's Jacobian index arrays
  for the 'approximate' Jacobian type (same four mechanisms);
* ``synthetic_small.inp``: the seeded all-forms synthetic mechanism.
"""
import argparse
import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

SOURCES = {
    "h2o2": ("data/h2o2.inp", None),
    "gri30": ("data/grimech30.inp", "data/thermo30.dat"),
    "testmech": ("tests/golden/test_mech.inp", None),
    "synthetic_small": ("tests/golden/synthetic_small.inp", None),
}


def flatten(val, prefix=""):
    out = {}
    for k, v in val.items():
        key = prefix + k
        if isinstance(v, dict):
            out.update(flatten(v, key + "/"))
        elif isinstance(v, (list, tuple)):
            if len(v) and isinstance(v[0], (list, tuple, np.ndarray)):
                for i, x in enumerate(v):
                    out["%s#%d" % (key, i)] = np.asarray(x, dtype=np.float64)
            else:
                out[key] = np.asarray(v)
        elif v is None:
            out[key] = np.asarray(np.nan)
        elif isinstance(v, np.ndarray) and v.dtype == object:
            for i, x in enumerate(v):
                out["%s#%d" % (key, i)] = np.asarray(x, dtype=np.float64)
        else:
            out[key] = np.asarray(v)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None)
    a = ap.parse_args()
    build_ref = importlib.import_module("build_ref")
    a.reference = build_ref.reference_dir(a.reference)
    rf = importlib.import_module("ref_frontend")
    conftest = importlib.import_module("conftest")
    syn = importlib.import_module("pyjac-v2_gb300.mech.synthetic")
    syn.write(os.path.join(HERE, "synthetic_small.inp"), **conftest.SYNTHETIC_SMALL)
    for name, (mech, therm) in SOURCES.items():
        specs, reacs, val = rf.reference_tables(os.path.join(ROOT, mech),
                                                os.path.join(ROOT, therm) if therm else None,
                                                reference=a.reference)
        flat = flatten(val)
        flat["species_names"] = np.array([s.name for s in specs])
        flat["reaction_strings"] = np.array([r.rxn_str for r in reacs])
        np.savez_compressed(os.path.join(HERE, "tables_%s.npz" % name), **flat)
        # the 'approximate' Jacobian type's index arrays (create_jacobian.py:186-190)
        _, _, aval = rf.reference_tables(os.path.join(ROOT, mech),
                                         os.path.join(ROOT, therm) if therm else None,
                                         jac_type="approximate", reference=a.reference)
        np.savez_compressed(os.path.join(HERE, "jacapprox_%s.npz" % name),
                            **flatten(aval["jac_inds"]))
    build_ref.build(a.reference, quiet=True)
    orc = importlib.import_module("oracle")
    states = importlib.import_module("pyjac-v2_gb300.states")
    for name, shipped, n, floor in (("h2o2", "h2o2", 256, None), ("gri30", "ch4", 1024, 1e-12)):
        ref = orc.RefKernels(shipped)
        P, phi = states.draw_states(ref.ns, n, seed=2024, x_floor=floor)
        phiF = np.ascontiguousarray(phi.T)
        dphi = ref.species_rates_F(P, phiF, nthreads=1)
        jac = ref.jacobian_F(P, phiF, nthreads=1)
        # species thermo (chem_utils) over a temperature sweep through both
        # NASA ranges and beyond the 100 K / 10,000 K guard
        cu_phi = np.repeat(phi[:1], 256, axis=0)
        cu_phi[:, 0] = np.linspace(50.0, 12000.0, 256)
        cp, h, b = ref.chem_utils_F(np.ascontiguousarray(cu_phi.T), nthreads=1)
        np.savez_compressed(os.path.join(HERE, "ref_%s.npz" % name), P=P, phi=phi,
                            dphi_F=dphi, jac_F=jac, cu_phi=cu_phi, cu_cp_F=cp, cu_h_F=h,
                            cu_b_F=b)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()

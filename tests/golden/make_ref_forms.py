"""Golden values for the rate forms no shipped reference kernel covers: PLOG,
Chebyshev, SRI (and Troe) fall-off blending, and the temperature and
extra-variable rates at constant volume as well as constant pressure.

The values come from the reference's own kernel text: its generators
(pyjac/core/rate_subs.py get_plog_arrhenius_rates :2084,
get_cheb_arrhenius_rates :1904, get_sri_kernel :2472, get_troe_kernel :2350,
get_temperature_rate :963, get_extra_var_rates :798) run unmodified under the
stub-import harness (oracle/ref_frontend.py) on the reference's all-forms test
mechanism (tests/golden/test_mech.inp), and the loopy instruction text they
emit is executed by oracle/loopy_eval.py for each state.  The kernels' inputs
that other sub-kernels produce (reduced pressures, concentrations, net rates,
specific heats and enthalpies, dT/dt) are taken from the oracle and stored
beside the outputs, so each formula is pinned on its own.

    python tests/golden/make_ref_forms.py [--reference DIR]

writes tests/golden/ref_forms_testmech.npz.  Needs the reference tree
(--reference, else PYJAC_REFERENCE, else the default of oracle/build_ref.py).
"""
import argparse
import importlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

MECH = os.path.join(HERE, "test_mech.inp")
OUT = os.path.join(HERE, "ref_forms_testmech.npz")
N = 48
SEED = 11


def states(mech, conp):
    st = importlib.import_module("pyjac-v2_gb300.states")
    # temperatures through both NASA ranges and beyond the 100 K / 10,000 K
    # guards, pressures around and outside the PLOG / Chebyshev tables
    P, phi = st.draw_states(mech.n_species, N, seed=SEED + (0 if conp else 1), x_floor=1e-12,
                            conp=conp, T_range=(300.0, 3000.0), p_atm_range=(0.01, 200.0))
    phi[:4, 0] = (50.0, 150.0, 9000.0, 12000.0)
    return P, phi


def run_forms(ref_kernels, info, mech, o, conp):
    le = importlib.import_module("loopy_eval")
    P, phi = states(mech, conp)
    d = o.rates_detail(P, phi, conp=conp)
    cp, h, _ = o.chem_utils(phi, conp=conp)
    n, ns, nn = phi.shape[0], mech.n_species, mech.nn
    pres = P if conp else phi[:, 1]  # the pressure of each state
    out = {"P": P, "phi": phi, "in_Pr": d["Pr"], "in_conc": d["conc"], "in_wdot": d["wdot"],
           "in_cp": cp, "in_h": h, "in_Tdot": d["dphi"][:, 0]}
    fall = info["fall"]
    for name, knl in ref_kernels.items():
        if name == "plog":
            n_loop, res = int(info["plog"]["num"]), np.zeros((n, int(info["plog"]["num"])))
            pp = info["plog"]["post_process"]
            base = {"plog_params": np.asarray(pp["params"]), "plog_num_param": np.asarray(info["plog"]["num_P"]),
                    "low": np.zeros(4), "hi": np.zeros(4)}
        elif name == "cheb":
            n_loop, res = int(info["cheb"]["num"]), np.zeros((n, int(info["cheb"]["num"])))
            pp = info["cheb"]["post_process"]
            base = {"cheb_Plim": np.asarray(pp["Plim"]), "cheb_Tlim": np.asarray(pp["Tlim"]),
                    "cheb_numP": np.asarray(info["cheb"]["num_P"]),
                    "cheb_numT": np.asarray(info["cheb"]["num_T"]),
                    "cheb_params": np.asarray(pp["params"], dtype=np.float64),
                    "cheb_pres_poly": np.zeros(16), "cheb_temp_poly": np.zeros(16)}
        elif name in ("sri", "troe"):
            sub = fall[name]
            n_loop = int(sub["num"])
            res = np.zeros((n, d["Pr"].shape[1]))
            base = {"%s_%s" % (name, k): np.asarray(sub[k], dtype=np.float64)
                    for k in (("a", "b", "c", "d", "e") if name == "sri" else ("a", "T1", "T2", "T3"))}
            base.update({"Pr": d["Pr"], "Fi": res, "X": np.zeros((n, n_loop)),
                         "Fcent": np.zeros((n, n_loop)), "Atroe": np.zeros((n, n_loop)),
                         "Btroe": np.zeros((n, n_loop))})
        elif name == "temperature":
            n_loop, res = ns, np.zeros((n, nn))
            base = {"wdot": d["wdot"], "conc": d["conc"], "dphi": res,
                    ("h" if conp else "u"): h, ("cp" if conp else "cv"): cp}
        else:  # extra_var
            n_loop, res = ns - 1, np.zeros((n, nn))
            res[:, 0] = d["dphi"][:, 0]
            base = {"wdot": d["wdot"], "dphi": res, "mw_factor": np.asarray(info["mw_post"])}
        for j in range(n):
            env = dict(base, j=j, phi=phi, P_arr=pres, V_arr=(phi[:, 1] if conp else P))
            if name in ("plog", "cheb"):
                kf = np.zeros((n, n_loop))
                env["kf"] = kf
                le.run(knl, env, n_loop)
                res[j] = kf[j]
            else:
                le.run(knl, env, n_loop)
        out["ref_" + name] = res.copy()
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None)
    a = ap.parse_args()
    ref_dir = importlib.import_module("build_ref").reference_dir(a.reference)
    rf = importlib.import_module("ref_frontend")
    orc = importlib.import_module("oracle")
    mech = importlib.import_module("pyjac-v2_gb300").load_mechanism(MECH)
    o = orc.Oracle(mech)
    res = {}
    for conp in (True, False):
        knls, info, _ = rf.reference_rate_kernels(MECH, conp=conp, reference=ref_dir)
        tag = "conp" if conp else "conv"
        for k, v in run_forms(knls, info, mech, o, conp).items():
            res["%s/%s" % (tag, k)] = v
        res["%s/texts" % tag] = np.array(["%s\n%s" % (k, knls[k].instructions) for k in sorted(knls)])
    res["plog_map"] = np.asarray(info["plog"]["map"])
    res["cheb_map"] = np.asarray(info["cheb"]["map"])
    res["sri_map"] = np.asarray(info["fall"]["sri"]["map"])
    res["troe_map"] = np.asarray(info["fall"]["troe"]["map"])
    np.savez_compressed(OUT, **res)
    print("written", OUT)


if __name__ == "__main__":
    main()

"""Front end parity (CPU): Chemkin reader, pyJac tables and Jacobian index arrays.

Bit-exact against the reference front end's own output, stored in
tests/golden/tables_<mech>.npz by tests/golden/make_golden.py (and, where the
reference tree exists, against a live run of it).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, REFERENCE, MECH_FILES, load_mech, pkg

sys_names = ["h2o2", "gri30", "testmech", "synthetic_small"]


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


@pytest.mark.parametrize("name", sys_names)
def test_tables_bit_exact_vs_golden(name):
    mech = load_mech(name)
    gold = np.load(os.path.join(GOLDEN, "tables_%s.npz" % name))
    mine = flatten(mech.val)
    keys = [k for k in gold.files if k not in ("species_names", "reaction_strings")]
    assert set(keys) == set(mine), sorted(set(keys) ^ set(mine))
    for k in keys:
        a, b = gold[k], mine[k]
        if a.dtype.kind == "f" and a.ndim == 0 and np.isnan(a):
            assert b.dtype.kind == "f" and np.isnan(b), k
            continue
        assert a.shape == b.shape, k
        assert a.dtype == b.dtype or (a.size == 0 and b.size == 0), (k, a.dtype, b.dtype)
        assert np.array_equal(a, b), k
    assert list(gold["species_names"]) == mech.species_names()
    assert list(gold["reaction_strings"]) == mech.reaction_strings()


def test_gri_index_arrays_match_shipped_header():
    """GRI-30 CCS pattern: nnz 1984, col_ptr as in the shipped jacobian.oclh."""
    mech = load_mech("gri30")
    ptr, ind = mech.pattern("F")
    assert mech.jac_nnz() == 1984 and ptr[-1] == 1984
    assert list(ptr[:8]) == [0, 53, 106, 156, 209, 259, 303, 356]
    # the bath gas N2 is last; AR (no reactions) has an empty row
    assert mech.species_names()[-1] == "N2"
    assert 49 not in set(ind[ptr[0]:ptr[1]])


def test_crs_ccs_consistent():
    for name in sys_names:
        mech = load_mech(name)
        rp, ci = mech.pattern("C")
        cp, ri = mech.pattern("F")
        nn = mech.nn
        dense_c = np.zeros((nn, nn), bool)
        dense_f = np.zeros((nn, nn), bool)
        for r in range(nn):
            dense_c[r, ci[rp[r]:rp[r + 1]]] = True
            dense_f[ri[cp[r]:cp[r + 1]], r] = True
        assert np.array_equal(dense_c, dense_f)
        assert dense_c[0].all() and dense_c[1].all()


@pytest.mark.skipif(not os.path.isdir(os.path.join(REFERENCE, "pyjac")), reason="reference tree absent")
def test_live_reference_frontend_matches():
    import sys
    sys.path.insert(0, os.path.join(os.path.dirname(GOLDEN), "..", "oracle"))
    rf = pytest.importorskip("ref_frontend")
    for name in ("h2o2", "gri30", "testmech"):
        mech_f, therm = MECH_FILES[name]
        specs, reacs, val = rf.reference_tables(mech_f, therm)
        mine = flatten(load_mech(name).val)
        ref = flatten(val)
        for k in ref:
            a, b = np.asarray(ref[k]), np.asarray(mine[k])
            assert np.array_equal(a, b, equal_nan=a.dtype.kind == "f") or (
                a.size == 0 and b.size == 0), (name, k)


def test_last_species_override_and_default():
    pj = pkg()
    f = MECH_FILES["gri30"]
    m = pj.load_mechanism(f[0], f[1], last_spec="AR")
    assert m.species_names()[-1] == "AR"
    m2 = pj.load_mechanism(f[0], f[1], last_spec="not-a-species")
    assert m2.species_names()[-1] == "N2"


def test_rev_parameters_split_into_two_reactions(tmp_path):
    text = """ELEMENTS H O
END
SPECIES H O OH
END
REACTIONS
H + O <=> OH  1.0E13 0.0 1000.0
  REV / 2.0E12 0.5 500.0 /
END
"""
    p = tmp_path / "m.inp"
    p.write_text(text)
    therm = os.path.join(os.path.dirname(GOLDEN), "..", "data", "thermo30.dat")
    m = pkg().load_mechanism(str(p), therm)
    assert m.n_reactions == 2
    assert all(" => " in s for s in m.reaction_strings())


def test_parser_errors(tmp_path):
    ck = pkg("mech.chemkin")
    bad = tmp_path / "bad.inp"
    bad.write_text("ELEMENTS H END\nSPECIES H END\nREACTIONS\nH + X <=> H  1.0 0.0 0.0\nEND\n")
    with pytest.raises(ck.ChemkinError):
        ck.read_mech(str(bad), None)
    units = tmp_path / "units.inp"
    units.write_text("ELEMENTS H END\nSPECIES H END\nREACTIONS FURLONGS\nEND\n")
    with pytest.raises(ck.ChemkinError):
        ck.read_mech(str(units), None)


def test_synthetic_generator_deterministic_and_balanced():
    syn = pkg("mech.synthetic")
    a = syn.generate(n_species=30, n_reactions=60, seed=5)
    b = syn.generate(n_species=30, n_reactions=60, seed=5)
    assert a == b
    mech = load_mech("synthetic_small")
    mw = mech.mw
    for r in mech.reactions:
        lhs = sum(mw[s] * nu for s, nu in zip(r.reac, r.reac_nu))
        rhs = sum(mw[s] * nu for s, nu in zip(r.prod, r.prod_nu))
        assert abs(lhs - rhs) < 1e-9 * lhs
        assert mech.n_species - 1 not in r.reac + r.prod
    kinds = {r.kind for r in mech.reactions}
    ck = pkg("mech.chemkin")
    assert {ck.ELEMENTARY, ck.THD, ck.FALL, ck.PLOG, ck.CHEB} <= kinds


@pytest.mark.parametrize("name", ["h2o2", "gri30", "testmech", "synthetic_small"])
def test_approximate_jacobian_pattern_bit_exact_vs_golden(name):
    """The 'approximate' Jacobian type drops the full rows of reactions with the
    bath gas (create_jacobian.py:186-190); index arrays equal the reference
    front end's."""
    mech = load_mech(name, jac_type="approximate")
    gold = np.load(os.path.join(GOLDEN, "jacapprox_%s.npz" % name))
    mine = flatten(mech.val["jac_inds"])
    assert set(gold.files) == set(mine)
    for k in gold.files:
        assert np.array_equal(gold[k], mine[k]), k
    assert mech.jac_nnz() <= load_mech(name).jac_nnz()

"""The packed reaction order of the device tables (host logic, no GPU).

The evaluation kernels run reactions in groups, each compiled for its
stoichiometry: the elementary class A + B <=> C + D, ten mass-action
patterns without third body and three third-body / fall-off patterns, then
the general code for the rest.  pjg_reaction_order returns the library's
packing; here it is checked against a plain restatement of the rules on the
packed records of the mechanism: every reaction appears once, each group
holds exactly the reactions the rules assign to it, and the groups come in the
order the kernels run them.  Within the elementary and mass-action groups the
order is the mechanism's; within the third-body groups and the general group,
the later reactions whose [M] is the same function of the state as an
earlier one's (same default efficiency and (species, efficiency) list) are
moved up to follow it, every other reaction keeping its mechanism order, so
that the kernels form [M] and ln [M] once per list.
"""
import numpy as np
import pytest

from conftest import load_mech, pkg

# (reversible, canonical coefficients): reactant entries by coefficient,
# then entries on both sides, then product entries by coefficient
MA = [(False, [(1, 0), (1, 0), (0, 1), (0, 1), (0, 1)]),
      (True, [(1, 0), (1, 0), (0, 1), (0, 1), (0, 1)]),
      (True, [(1, 0), (1, 0), (0, 2)]),
      (True, [(2, 0), (0, 1), (0, 1)]),
      (True, [(1, 0), (1, 0), (1, 0), (0, 1), (0, 1)]),
      (True, [(1, 0), (1, 0), (0, 1), (0, 2)]),
      (True, [(1, 0), (2, 0), (0, 1), (0, 1)]),
      (False, [(1, 0), (1, 0), (0, 1), (0, 1)]),
      (True, [(1, 0), (1, 1), (0, 1)]),
      (True, [(1, 0), (1, 0), (1, 1), (0, 1)])]
TP = [(True, [(1, 0), (1, 0), (0, 1)]),
      (True, [(1, 0), (0, 1), (0, 1)]),
      (True, [(2, 0), (0, 1)])]


def _key(rec):
    """Reactant-only entries by coefficient, then entries on both sides, then
    product-only entries by coefficient; None with a coefficient above 2."""
    ents = [(int(e >> 16) & 0xFF, int(e >> 24)) for e in rec["ent"][:rec["nspec"]]]
    if any(max(f, r) > 2 for f, r in ents):
        return None
    return (sorted(x for x in ents if x[1] == 0) + sorted(x for x in ents if x[0] and x[1]) +
            sorted(x for x in ents if x[0] == 0))


def third_body_keys(tables):
    """Per reaction: the mechanism index of the first reaction with the same
    default efficiency and efficiency list, -1 without a third body."""
    seen, keys = {}, []
    for i, r in enumerate(tables.rxn):
        if (int(r["flags"]) >> 4) & 3 == 0:
            keys.append(-1)
            continue
        o, n = int(r["thd_off"]), int(r["thd_cnt"])
        k = (float(r["p"][12]),) + tuple((int(tables.thd_spec[o + l]), float(tables.thd_coef[o + l]))
                                         for l in range(n))
        keys.append(seen.setdefault(k, i))
    return np.array(keys)


def expected_class(rec):
    flags = int(rec["flags"])
    form, rev, thd = flags & 7, bool(flags & 8), (flags >> 4) & 3
    key = _key(rec)
    if form > 2 or key is None:
        return -1
    if (rec["nspec"] == 4 and rev and thd == 0 and rec["nu_sum"] == 0 and rec["p"][11] == 1.0
            and key == [(1, 0), (1, 0), (0, 1), (0, 1)]):
        return 0
    if thd == 0 and 3 <= rec["nspec"] <= 5:
        for q, (r, k) in enumerate(MA):
            if r == rev and k == key:
                return 1 + q
    if thd != 0:
        for t, (r, k) in enumerate(TP):
            if r == rev and k == key:
                return 1 + len(MA) + t
    return -1


@pytest.mark.parametrize("name", ["h2o2", "gri30", "testmech", "synthetic_small"])
def test_packing_matches_the_rules(name):
    mech = load_mech(name)
    orig, cls = pkg("api").reaction_order(mech)
    tables = pkg("pack").PackedTables(mech)
    rx = tables.rxn
    assert sorted(orig.tolist()) == list(range(len(rx)))
    want = np.array([expected_class(rx[i]) for i in orig])
    assert np.array_equal(cls, want)
    # groups in kernel order (elementary, patterns, general last)
    rank = np.where(cls < 0, 99, cls)
    assert np.all(np.diff(rank) >= 0)
    key = third_body_keys(tables)
    for g in np.unique(rank):
        members = orig[rank == g]
        if g <= 10:
            assert np.all(np.diff(members) > 0)   # mechanism order
        else:
            want, done = [], set()
            for i in sorted(members.tolist()):
                if i in done:
                    continue
                same = [j for j in sorted(members.tolist()) if key[i] >= 0 and key[j] == key[i]]
                for j in same or [i]:
                    want.append(j)
                    done.add(j)
            assert members.tolist() == want


def test_gri30_group_sizes():
    """GRI-Mech 3.0: 232 elementary reactions, 41 in the mass-action patterns,
    all 41 third-body and fall-off reactions in the third-body patterns, 11
    for the general code."""
    orig, cls = pkg("api").reaction_order(load_mech("gri30"))
    assert int((cls == 0).sum()) == 232
    assert int(((cls >= 1) & (cls <= 10)).sum()) == 41
    assert int(((cls >= 11) & (cls <= 13)).sum()) == 41
    assert int((cls == -1).sum()) == 11


RX_SAMEM, RX_SAMELNM = 1 << 20, 1 << 21


@pytest.mark.parametrize("name", ["h2o2", "gri30", "testmech", "synthetic_small"])
def test_third_body_reuse_marks(name):
    """RX_SAMEM marks a record whose [M] equals the previous record's (same
    third-body list key, same group), RX_SAMELNM one whose run of such records
    has already formed ln [M] (an earlier Troe or SRI fall-off whose two rate
    constants are both of the exponential form); the kernels reuse [M] and
    ln [M] exactly there."""
    mech = load_mech(name)
    orig, cls, flags = pkg("api").reaction_order(mech, with_flags=True)
    tables = pkg("pack").PackedTables(mech)
    key = third_body_keys(tables)
    run_log = False
    for q in range(len(orig)):
        f = int(flags[q])
        same = (q > 0 and key[orig[q]] >= 0 and key[orig[q]] == key[orig[q - 1]]
                and cls[q] == cls[q - 1])
        if not same:
            run_log = False
        assert bool(f & RX_SAMEM) == same
        assert bool(f & RX_SAMELNM) == (same and run_log)
        blend, thd = (f >> 6) & 3, (f >> 4) & 3
        if thd and blend in (2, 3) and f & 7 == 2 and (f >> 9) & 3 == 2:
            run_log = True
        # the marks aside, the flag word is the record's own
        assert f & ~(RX_SAMEM | RX_SAMELNM) == int(tables.rxn[orig[q]]["flags"])


def test_gri30_shares_third_body_concentrations():
    """GRI-Mech 3.0: 41 third-body and fall-off reactions, 11 distinct [M];
    the packing forms [M] for fewer than half of them."""
    orig, cls, flags = pkg("api").reaction_order(load_mech("gri30"), with_flags=True)
    thd = ((flags >> 4) & 3) != 0
    assert int(thd.sum()) == 41
    assert int((thd & ((flags & RX_SAMEM) == 0)).sum()) < 20

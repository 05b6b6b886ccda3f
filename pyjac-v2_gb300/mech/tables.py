"""Mechanism tables and Jacobian sparsity, with pyJac's exact field semantics.

``build_tables`` turns a parsed mechanism into the same per-reaction and
per-species tables as pyJac's ``assign_rates`` (pyjac/core/rate_subs.py:74-537)
and the same Jacobian non-zero pattern as ``determine_jac_inds``
(pyjac/core/create_jacobian.py:68-283).  Index tables are int32
(pyJac's ``kint_type``), parameters float64.  The dictionaries use the
reference's key names so that they can be compared entry by entry.

Species ordering follows ``find_last_species`` (create_jacobian.py:5131-5209):
the user's bath gas, else the first of N2 / Ar / He whose name and molecular
weight both match, is moved to the end; reaction species lists are then
re-indexed and sorted by species index (pyjac/utils.py:613-645).
"""
import numpy as np

from . import chemkin as ck
from .elements import atomic_weights

KINT = np.int32

# rate specialisation (rate_subs.py:86-103): 'full', 'hybrid' or 'fixed'
RATE_SPECS = ("fixed", "hybrid", "full")


def find_last_species(specs, last_spec=None):
    """Return the index of the species to move to the end (create_jacobian.py:5131)."""
    if last_spec is not None:
        want = last_spec.lower().strip()
        for i, sp in enumerate(specs):
            if sp.name.lower() == want:
                return i
    wt = atomic_weights()
    for name, mw in (('N2', wt['n'] * 2.), ('Ar', wt['ar']), ('He', wt['he'])):
        for i, sp in enumerate(specs):
            if sp.name.lower() == name.lower() and sp.mw == mw:
                return i
    return len(specs) - 1


def reorder(specs, reacs, last_spec=None):
    """Move the bath gas last and turn reaction species into sorted indices."""
    specs = list(specs)
    specs.append(specs.pop(find_last_species(specs, last_spec)))
    index = {sp.name: i for i, sp in enumerate(specs)}
    for r in reacs:
        pairs = sorted(zip(r.reac, r.reac_nu), key=lambda x: index[x[0]])
        r.reac = [index[s] for s, _ in pairs]
        r.reac_nu = [nu for _, nu in pairs]
        pairs = sorted(zip(r.prod, r.prod_nu), key=lambda x: index[x[0]])
        r.prod = [index[s] for s, _ in pairs]
        r.prod_nu = [nu for _, nu in pairs]
        r.thd_body_eff = sorted([(index[t[0]], t[1]) for t in r.thd_body_eff],
                                key=lambda x: x[0])
        r.pdep_sp = index[r.pdep_sp] if r.pdep_sp != '' else None
    return specs, reacs


def _net_nu(isp, r):
    """Net stoichiometric coefficient of species isp (pyjac/utils.py:516-545)."""
    if isp in r.prod and isp in r.reac:
        nu = r.prod_nu[r.prod.index(isp)] - r.reac_nu[r.reac.index(isp)]
        if nu == 0:
            return 0
    elif isp in r.prod:
        nu = r.prod_nu[r.prod.index(isp)]
    elif isp in r.reac:
        nu = -r.reac_nu[r.reac.index(isp)]
    else:
        return 0
    return nu


def _offsets(counts):
    counts = np.asarray(counts, dtype=np.int64)
    return np.concatenate((np.cumsum(counts) - counts, [counts.sum()])).astype(KINT)


def _is_int(v):
    return float(v).is_integer()


def _stack(arrays):
    """np.array of equally shaped arrays; an object array when they are ragged."""
    try:
        return np.array(arrays)
    except ValueError:
        out = np.empty(len(arrays), dtype=object)
        for i, a in enumerate(arrays):
            out[i] = a
        return out


def _specialize(rates, rate_spec, fall=False):
    """Per-reaction Arrhenius parameters and rate type (rate_subs.py:219-266)."""
    n = len(rates)
    rtype = np.zeros(n, dtype=KINT)
    ftype = np.zeros(n, dtype=KINT) if fall else None
    A = np.zeros(n)
    b = np.zeros(n)
    Ta = np.zeros(n)
    for i, r in enumerate(rates):
        if fall and (r.high or r.low):
            if r.high:
                Ai, bi, Ti = r.high
                ftype[i] = 1        # chemically activated
            else:
                Ai, bi, Ti = r.low
                ftype[i] = 0        # fall-off (k0 is the "other" rate)
        else:
            Ai, bi, Ti = r.A, r.b, r.E
        A[i] = np.log(Ai)
        b[i] = bi
        Ta[i] = Ti
        if rate_spec == "fixed":
            rtype[i] = 0
            continue
        if bi == 0 and Ti == 0:
            A[i] = Ai
            rtype[i] = 0
        elif bi == int(bi) and bi and Ti == 0:
            A[i] = Ai
            rtype[i] = 1
        elif Ti == 0 and bi != 0:
            rtype[i] = 2
        elif bi == 0 and Ti != 0:
            rtype[i] = 3
        else:
            rtype[i] = 4
        if rate_spec != "full":
            rtype[i] = rtype[i] if rtype[i] <= 1 else 2
    return rtype, A, b, Ta, ftype


def assign_rates(reacs, specs, rate_spec="hybrid"):
    """pyJac's mechanism tables (rate_subs.py:74-537), as a dict of numpy arrays."""
    if rate_spec not in RATE_SPECS:
        raise ValueError("rate_spec must be one of %s" % (RATE_SPECS,))
    Ns = len(specs)
    last = Ns - 1
    rev_map = np.array([i for i, r in enumerate(reacs) if r.rev], dtype=KINT)

    nu_sum, net_num, net_spec, net_nu, has_ns, ns_nu = [], [], [], [], [], []
    for i, r in enumerate(reacs):
        slist = sorted(set(r.reac + r.prod))
        net_spec.extend(slist)
        net_num.append(len(slist))
        for s in slist:
            rn = r.reac_nu[r.reac.index(s)] if s in r.reac else 0
            pn = r.prod_nu[r.prod.index(s)] if s in r.prod else 0
            net_nu.extend([pn, rn])
        nu_sum.append(sum(_net_nu(s, r) for s in slist))
        rn = r.reac_nu[r.reac.index(last)] if last in r.reac else 0
        pn = r.prod_nu[r.prod.index(last)] if last in r.prod else 0
        if rn or pn:
            has_ns.append(i)
            ns_nu.extend([pn, rn])
    allint = all(_is_int(v) for v in net_nu)
    fdt = KINT if allint else np.float64
    net = {"num_reac_to_spec": np.array(net_num, dtype=KINT),
           "nu_sum": np.array(nu_sum, dtype=fdt),
           "nu": np.array(net_nu, dtype=fdt),
           "reac_to_spec": np.array(net_spec, dtype=KINT),
           "allint": allint}

    s2r, snu, scount, slist = [], [], [], []
    for isp in range(Ns):
        lst = [(i, _net_nu(isp, r)) for i, r in enumerate(reacs)]
        lst = [x for x in lst if x[1]]
        if lst:
            s2r.extend(x[0] for x in lst)
            snu.extend(x[1] for x in lst)
            scount.append(len(lst))
            slist.append(isp)
    per_spec = {"reac_count": np.array(scount, dtype=KINT),
                "nu": np.array(snu, dtype=fdt),
                "reacs": np.array(s2r, dtype=KINT),
                "map": np.array(slist, dtype=KINT), "allint": allint}

    def separate(kinds):
        idx = [i for i, r in enumerate(reacs) if r.kind in kinds]
        return [reacs[i] for i in idx], np.array(idx, dtype=KINT), len(idx)

    simple, simple_map, n_simple = separate((ck.ELEMENTARY, ck.THD, ck.FALL, ck.CHEM))
    s_type, s_A, s_b, s_Ta, _ = _specialize(simple, rate_spec)

    plog, plog_map, n_plog = separate((ck.PLOG,))
    num_P = np.array([len(r.plog_par) for r in plog], dtype=KINT)
    plog_params = [r.plog_par for r in plog]
    pp_plog = np.empty(0)
    maxP = None
    if n_plog:
        maxP = num_P.max()
        pp_plog = np.zeros((4, n_plog, int(maxP)))
        for m in range(4):
            for i, nP in enumerate(num_P):
                for j in range(nP):
                    pp_plog[m, i, j] = plog_params[i][j][m]
        with np.errstate(divide="ignore"):
            pp_plog[0] = np.log(pp_plog[0])
            pp_plog[1] = np.log(pp_plog[1])
        pp_plog[np.isinf(pp_plog)] = 0

    cheb, cheb_map, n_cheb = separate((ck.CHEB,))
    cheb_nP = np.array([r.cheb_n_pres for r in cheb], dtype=KINT)
    cheb_nT = np.array([r.cheb_n_temp for r in cheb], dtype=KINT)
    cheb_plim = np.array([r.cheb_plim for r in cheb])
    cheb_tlim = np.array([r.cheb_tlim for r in cheb])
    pp_cheb = np.empty(0)
    pp_cheb_plim = np.empty(0)
    pp_cheb_tlim = np.empty(0)
    if n_cheb:
        pp_cheb = np.zeros((n_cheb, int(cheb_nT.max()), int(cheb_nP.max())))
        for i, r in enumerate(cheb):
            pp_cheb[i, :cheb_nT[i], :cheb_nP[i]] = np.array(r.cheb_par, dtype=np.float64)
        pp_cheb_plim = np.log(np.array(cheb_plim, dtype=np.float64))
        pp_cheb_tlim = 1. / np.array(cheb_tlim, dtype=np.float64)

    fall, fall_map, n_fall = separate((ck.FALL, ck.CHEM))
    f_type, f_A, f_b, f_Ta, f_ftype = _specialize(fall, rate_spec, fall=True)
    blend = np.array([r.fall_form for r in fall], dtype=KINT)
    lind_map = np.where(blend == ck.FALL_LIND)[0].astype(KINT)
    sri_map = np.where(blend == ck.FALL_SRI)[0].astype(KINT)
    sri_par = [list(reacs[fall_map[i]].sri_par) for i in sri_map]
    for p in sri_par:
        if len(p) != 5:
            p.extend([1, 0])
    if sri_par:
        sri_a, sri_b, sri_c, sri_d, sri_e = [np.array(x, dtype=np.float64) for x in zip(*sri_par)]
    else:
        sri_a = sri_b = sri_c = sri_d = sri_e = np.empty(0)
    troe_map = np.where(blend == ck.FALL_TROE)[0].astype(KINT)
    troe_par = [list(reacs[fall_map[i]].troe_par) for i in troe_map]
    for p in troe_par:
        if len(p) != 4:
            p.append(0)
    if troe_par:
        troe_a, troe_T3, troe_T1, troe_T2 = [np.array(x, dtype=np.float64) for x in zip(*troe_par)]
        troe_T1 = 1. / troe_T1
        troe_T3 = 1. / troe_T3
    else:
        troe_a = troe_T3 = troe_T1 = troe_T2 = np.empty(0)

    thd, thd_map, n_thd = separate((ck.FALL, ck.CHEM, ck.THD))
    thd_type = np.array([r.thd_kind for r in thd], dtype=KINT)
    t_num, t_spec, t_eff, t_has_ns, t_ns_eff = [], [], [], [], []
    for i, r in enumerate(thd):
        if r.thd_kind == ck.THD_SPECIES:
            t_num.append(1)
            t_spec.append(r.pdep_sp)
            t_eff.append(1)
            if r.pdep_sp == last:
                t_has_ns.append(i)
                t_ns_eff.append(1)
        elif r.thd_kind == ck.THD_UNITY:
            t_num.append(0)
        else:
            t_num.append(len(r.thd_body_eff))
            sp, eff = zip(*r.thd_body_eff)
            t_spec.extend(sp)
            t_eff.extend(eff)
            if last in sp:
                t_has_ns.append(i)
                t_ns_eff.append(eff[sp.index(last)])

    a_lo = np.zeros((Ns, 7))
    a_hi = np.zeros((Ns, 7))
    T_mid = np.zeros(Ns)
    for i, s in enumerate(specs):
        a_lo[i, :] = s.lo
        a_hi[i, :] = s.hi
        T_mid[i] = s.Trange[1]
    mws = np.array([s.mw for s in specs])
    minT = maxT = None
    for s in specs:
        minT = s.Trange[0] if minT is None else np.maximum(minT, s.Trange[0])
        maxT = s.Trange[-1] if maxT is None else np.minimum(maxT, s.Trange[-1])

    return {"simple": {"A": s_A, "b": s_b, "Ta": s_Ta, "type": s_type,
                       "num": n_simple, "map": simple_map},
            "plog": {"map": plog_map, "num": n_plog, "num_P": num_P,
                     "params": plog_params, "max_P": maxP,
                     "post_process": {"params": pp_plog}},
            "cheb": {"map": cheb_map, "num": n_cheb, "num_P": cheb_nP, "num_T": cheb_nT,
                     "params": _stack([np.array(r.cheb_par, dtype=np.float64) for r in cheb]),
                     "Tlim": cheb_tlim, "Plim": cheb_plim,
                     "post_process": {"params": pp_cheb, "Plim": pp_cheb_plim,
                                      "Tlim": pp_cheb_tlim}},
            "fall": {"map": fall_map, "num": n_fall, "ftype": f_ftype, "blend": blend,
                     "A": f_A, "b": f_b, "Ta": f_Ta, "type": f_type,
                     "sri": {"map": sri_map, "num": sri_map.size, "a": sri_a, "b": sri_b,
                             "c": sri_c, "d": sri_d, "e": sri_e},
                     "troe": {"map": troe_map, "num": troe_map.size, "a": troe_a,
                              "T3": troe_T3, "T1": troe_T1, "T2": troe_T2},
                     "lind": {"map": lind_map, "num": lind_map.size}},
            "thd": {"map": thd_map, "num": n_thd, "type": thd_type,
                    "spec_num": np.array(t_num, dtype=KINT),
                    "spec": np.array(t_spec, dtype=KINT),
                    "eff": np.array(t_eff, dtype=np.float64),
                    "has_ns": np.array(t_has_ns, dtype=KINT),
                    "eff_ns": np.array(t_ns_eff, dtype=np.float64)},
            "fwd": {"map": np.arange(len(reacs)), "num": len(reacs)},
            "rev": {"map": rev_map, "num": len(rev_map)},
            "net": net,
            "net_per_spec": per_spec,
            "Nr": len(reacs), "Ns": Ns,
            "thermo": {"a_lo": a_lo, "a_hi": a_hi, "T_mid": T_mid},
            "mws": mws, "mw_post": mws[:-1] / mws[-1],
            "reac_has_ns": np.array(has_ns, dtype=KINT),
            "ns_nu": np.array(ns_nu, dtype=fdt),
            "minT": minT, "maxT": maxT}


def jacobian_pattern(val, jac_type="exact"):
    """Non-zero (row, col) pattern of the Jacobian (create_jacobian.py:106-283).

    Rows/cols: 0 = temperature, 1 = extra variable, 2 + k = species k
    (k < Ns - 1).  Returns flat C / F index lists and CRS / CCS arrays.
    """
    Ns = val["Ns"]
    NN = Ns + 1
    so = 2
    inds = [(0, x) for x in range(NN)] + [(1, x) for x in range(NN)]
    nz_specs = val["net_per_spec"]["map"]
    rxn_count = _offsets(val["net_per_spec"]["reac_count"])
    rxn_maps = val["net_per_spec"]["reacs"]
    r2s = val["net"]["reac_to_spec"]
    nspec_off = _offsets(val["net"]["num_reac_to_spec"])
    has_ns = set(int(x) for x in val["reac_has_ns"])
    thd_has_ns = set(int(x) for x in val["thd"]["has_ns"])
    thd_spec = val["thd"]["spec"]
    thd_eff = val["thd"]["eff"]
    thd_index = {int(r): i for i, r in enumerate(val["thd"]["map"])}
    rev = set(int(x) for x in val["rev"]["map"])
    nu = val["net"]["nu"]
    thd_off = _offsets(val["thd"]["spec_num"])
    ns = Ns - 1
    for ii, spec in enumerate(nz_specs):
        if spec == Ns - 1:
            continue
        row = spec + so
        derivs = {0, 1}

        def add(lst):
            derivs.update(x + so for x in lst if x + so < NN)

        for rxn in rxn_maps[rxn_count[ii]:rxn_count[ii + 1]]:
            rxn = int(rxn)
            ti = thd_index.get(rxn)
            if (rxn in has_ns or (ti is not None and ti in thd_has_ns)) and jac_type != "approximate":
                add(range(NN))
                break
            dspecs = [int(x) for x in r2s[nspec_off[rxn]:nspec_off[rxn + 1]]]
            if rxn not in rev:
                nus = nu[2 * nspec_off[rxn]:2 * nspec_off[rxn + 1]]
                is_prod = [nus[2 * i] != 0 for i in range(len(dspecs))]
                is_reac = [nus[2 * i + 1] != 0 for i in range(len(dspecs))]
                k = dspecs.index(int(spec))
                if not (is_prod[k] and is_reac[k]):
                    dspecs = [x for i, x in enumerate(dspecs) if is_reac[i]]
            add(dspecs)
            if ti is not None:
                last_eff = 1.0
                tsp = thd_spec[thd_off[ti]:thd_off[ti + 1]]
                teff = thd_eff[thd_off[ti]:thd_off[ti + 1]]
                if ns in tsp:
                    last_eff = teff[list(tsp).index(ns)]
                add([int(x) for i, x in enumerate(tsp) if teff[i] != last_eff])
        inds.extend((row, x) for x in sorted(derivs))

    rows = np.array([r for r, _ in inds], dtype=KINT)
    cols = np.array([c for _, c in inds], dtype=KINT)
    order_F = np.lexsort((rows, cols))  # stable: by column, rows ascending
    flat_F = np.stack((rows[order_F], cols[order_F]), axis=1).astype(KINT)
    row_ptr = _offsets(np.bincount(rows, minlength=NN))
    col_ptr = _offsets(np.bincount(cols, minlength=NN))
    return {"flat_C": np.stack((rows, cols), axis=1).astype(KINT),
            "flat_F": flat_F,
            "crs": {"col_ind": cols.copy(), "row_ptr": row_ptr},
            "ccs": {"row_ind": rows[order_F].copy(), "col_ptr": col_ptr}}


def determine_jac_inds(reacs, specs, rate_spec="hybrid", jac_type="exact"):
    """assign_rates + sparsity, as create_jacobian.determine_jac_inds returns."""
    val = assign_rates(reacs, specs, rate_spec)
    val["jac_inds"] = jacobian_pattern(val, jac_type)
    return val

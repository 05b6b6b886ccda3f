"""Seeded synthetic large mechanism, emitted as Chemkin text.

Species are C_iH_j compositions plus an N2 bath gas, so every reaction
conserves elements and mass (the Jacobian's T and extra-variable rows use
sum_k W_k wdot_k = 0, as pyJac's do: create_jacobian.py dTdot_dnj :3382).
Reactions: 1-3 reactants and 1-3 products with coefficients 1-2, all
reversible, the bath gas in none of them and with default efficiency, so that
Jacobian rows stay sparse (create_jacobian.py:186-190).

Defaults follow the large-mechanism configuration: 500 species, 2500
reactions; A log-uniform in [1e6, 1e14] (cm-mol-s), b uniform in [-2, 2],
Ea uniform in [0, 50] kcal/mol; 10% third-body, 5% Troe, 2% SRI, 3% PLOG
(4 pressures), 1% Chebyshev (6 x 4); NASA-7 fits of smooth random cp(T) on
300-1000 K and 1000-3500 K, continuous (cp, h, s) at 1000 K.
"""
import numpy as np

from .elements import RU, atomic_weights


def _species_list(n_species, rng):
    comps = [(i, j) for i in range(0, 26) for j in range(0, 26) if i + j > 0]
    rng.shuffle(comps)
    comps = sorted(comps[:n_species - 1], key=lambda c: (c[0] + c[1], c))
    return comps


def _name(c):
    i, j = c
    return "C%dH%d" % (i, j) if i and j else ("C%d" % i if i else "H%d" % j)


def _nasa_fit(rng, mw):
    """Random smooth cp/R(T) fitted by NASA-7 polynomials, continuous at 1000 K."""
    Tlo = np.linspace(300.0, 1000.0, 40)
    Thi = np.linspace(1000.0, 3500.0, 60)
    nat = max(2.0, mw / 7.0)
    c_lo = 2.5 + 0.5 * nat * rng.uniform(0.3, 1.0)
    c_hi = c_lo + nat * rng.uniform(0.5, 2.0)
    Tm = rng.uniform(600.0, 1800.0)
    w = rng.uniform(300.0, 900.0)

    def cp(T):
        return c_lo + (c_hi - c_lo) * 0.5 * (1.0 + np.tanh((T - Tm) / w))

    def basis(T):
        return np.stack([np.ones_like(T), T, T ** 2, T ** 3, T ** 4], axis=1)

    # constrained least squares: same cp value at 1000 K from both fits
    def fit(T):
        return np.linalg.lstsq(basis(T), cp(T), rcond=None)[0]

    lo = fit(Tlo)
    hi = fit(Thi)
    b1000 = basis(np.array([1000.0]))[0]
    hi[0] += b1000 @ lo - b1000 @ hi
    hf = rng.uniform(-60000.0, 60000.0)      # h/R at 298 K-ish reference, K
    s0 = rng.uniform(20.0, 60.0)             # s/R offset

    def h_poly(a, T):
        return a[0] * T + a[1] * T ** 2 / 2 + a[2] * T ** 3 / 3 + a[3] * T ** 4 / 4 + a[4] * T ** 5 / 5

    def s_poly(a, T):
        return a[0] * np.log(T) + a[1] * T + a[2] * T ** 2 / 2 + a[3] * T ** 3 / 3 + a[4] * T ** 4 / 4

    a5_lo = hf - h_poly(lo, 298.15)
    a6_lo = s0 - s_poly(lo, 298.15)
    a5_hi = a5_lo + h_poly(lo, 1000.0) - h_poly(hi, 1000.0)
    a6_hi = a6_lo + s_poly(lo, 1000.0) - s_poly(hi, 1000.0)
    return list(lo) + [a5_lo, a6_lo], list(hi) + [a5_hi, a6_hi]


def _fmt(x):
    return "%.8E" % x


def _thermo_entry(name, comp, lo, hi):
    i, j = comp
    el = ""
    if i:
        el += "%-2s%3d" % ("C", i)
    if j:
        el += "%-2s%3d" % ("H", j)
    el = el.ljust(20)
    # columns: name 0:18, element block 24:44, phase 44, temperatures 45:74
    head = ("%-24s" % name)[:24] + el + "G" + "%10.3f%10.3f%9.3f" % (300.0, 3500.0, 1000.0)
    head = head.ljust(79) + "1\n"
    l2 = "".join("%15.8E" % x for x in hi[0:5]) + "    2\n"
    l3 = "".join("%15.8E" % x for x in (hi[5], hi[6], lo[0], lo[1], lo[2])) + "    3\n"
    l4 = "".join("%15.8E" % x for x in (lo[3], lo[4], lo[5], lo[6])) + "                   4\n"
    return head + l2 + l3 + l4


def _partition(total, comp_set, rng, max_parts=3, tries=200):
    """Random split of an (nC, nH) total into 1-3 species (with multiplicity)."""
    tc, th = total
    for _ in range(tries):
        k = rng.integers(1, max_parts + 1)
        if k == 1:
            if total in comp_set:
                return [total]
            continue
        cuts_c = sorted(rng.integers(0, tc + 1, size=k - 1))
        cuts_h = sorted(rng.integers(0, th + 1, size=k - 1))
        pc = np.diff([0] + list(cuts_c) + [tc])
        ph = np.diff([0] + list(cuts_h) + [th])
        parts = [(int(a), int(b)) for a, b in zip(pc, ph)]
        if all(p in comp_set for p in parts):
            return parts
    return None


def generate(n_species=500, n_reactions=2500, seed=0, frac_thd=0.10, frac_troe=0.05,
             frac_sri=0.02, frac_plog=0.03, frac_cheb=0.01, A_range=(1e6, 1e14),
             b_range=(-2.0, 2.0), Ea_kcal=(0.0, 50.0)):
    """Return Chemkin mechanism text (with THERMO section) for the synthetic mechanism."""
    rng = np.random.default_rng(seed)
    wt = atomic_weights()
    comps = _species_list(n_species, rng)
    comp_set = set(comps)
    names = [_name(c) for c in comps]
    mws = [c[0] * wt["c"] + c[1] * wt["h"] for c in comps]
    lines = ["ELEMENTS C H N END", "SPECIES"]
    allnames = names + ["N2"]
    for k in range(0, len(allnames), 8):
        lines.append("  " + " ".join(allnames[k:k + 8]))
    lines.append("END")
    lines.append("THERMO ALL")
    lines.append("   300.000  1000.000  3500.000")
    thermo = []
    for nm, c, mw in zip(names, comps, mws):
        lo, hi = _nasa_fit(rng, mw)
        thermo.append(_thermo_entry(nm, c, lo, hi))
    # N2 bath gas (smooth constant-ish cp)
    lo = [3.53100528, -1.23660988e-04, -5.02999433e-07, 2.43530612e-09, -1.40881235e-12,
          -1046.97628, 2.96747038]
    hi = [2.95257637, 1.39690040e-03, -4.92631603e-07, 7.86010195e-11, -4.60755204e-15,
          -923.948688, 5.87188762]
    n2 = ("%-24s" % "N2") + ("%-2s%3d" % ("N", 2)).ljust(20) + "G" + "%10.3f%10.3f%9.3f" % (300.0, 3500.0, 1000.0)
    n2 = n2.ljust(79) + "1\n"
    n2 += "".join("%15.8E" % x for x in hi[0:5]) + "    2\n"
    n2 += "".join("%15.8E" % x for x in (hi[5], hi[6], lo[0], lo[1], lo[2])) + "    3\n"
    n2 += "".join("%15.8E" % x for x in (lo[3], lo[4], lo[5], lo[6])) + "                   4\n"
    thermo.append(n2)
    body = "\n".join(lines) + "\n" + "".join(thermo) + "END\n"

    special = (["thd"] * int(round(frac_thd * n_reactions)) +
               ["troe"] * int(round(frac_troe * n_reactions)) +
               ["sri"] * int(round(frac_sri * n_reactions)) +
               ["plog"] * int(round(frac_plog * n_reactions)) +
               ["cheb"] * int(round(frac_cheb * n_reactions)))
    kinds = rng.permutation(special + ["el"] * max(0, n_reactions - len(special)))[:n_reactions]
    rx = ["REACTIONS"]
    made = 0
    guard = 0
    while made < n_reactions and guard < 100 * n_reactions:
        guard += 1
        kind = kinds[made]
        # fall-off and third-body reactions: at most two reactant species
        nreac = rng.integers(1, 3 if kind in ("troe", "sri", "thd") else 4)
        idx = rng.choice(len(comps), size=nreac, replace=False)
        nus = [int(rng.integers(1, 3)) for _ in idx]
        tot = (sum(comps[i][0] * nu for i, nu in zip(idx, nus)),
               sum(comps[i][1] * nu for i, nu in zip(idx, nus)))
        parts = _partition(tot, comp_set, rng)
        if parts is None:
            continue
        prod = {}
        for pc in parts:
            prod[pc] = prod.get(pc, 0) + 1
        if any(v > 2 for v in prod.values()) or len(prod) > 3:
            continue
        reac = {comps[i]: nu for i, nu in zip(idx, nus)}
        if reac == prod or len(set(reac) | set(prod)) > 8:
            continue
        order = sum(nus)
        if kind in ("troe", "sri") and order > 2:
            continue

        def side(d):
            return " + ".join(("%d%s" % (v, _name(c)) if v > 1 else _name(c)) for c, v in d.items())

        A = float(np.exp(rng.uniform(np.log(A_range[0]), np.log(A_range[1]))))
        b = float(rng.uniform(*b_range))
        Ea = float(rng.uniform(*Ea_kcal)) * 1000.0
        lhs, rhs = side(reac), side(prod)
        if kind == "el":
            rx.append("%s <=> %s  %s %.4f %.3f" % (lhs, rhs, _fmt(A), b, Ea))
        elif kind == "thd":
            rx.append("%s + M <=> %s + M  %s %.4f %.3f" % (lhs, rhs, _fmt(A / 10.0), b, Ea))
            effs = rng.choice(len(comps), size=3, replace=False)
            rx.append("  " + " ".join("%s/%.2f/" % (_name(comps[e]), rng.uniform(0.5, 5.0)) for e in effs))
        elif kind in ("troe", "sri"):
            rx.append("%s (+M) <=> %s (+M)  %s %.4f %.3f" % (lhs, rhs, _fmt(A), b, Ea))
            A0 = A * float(np.exp(rng.uniform(np.log(1e2), np.log(1e6))))
            rx.append("  LOW / %s %.4f %.3f /" % (_fmt(A0), float(rng.uniform(-3, 0)),
                                                  float(rng.uniform(0, 20)) * 1000.0))
            if kind == "troe":
                rx.append("  TROE / %.4f %.2f %.2f %.2f /" % (rng.uniform(0.2, 0.9), rng.uniform(50, 500),
                                                           rng.uniform(500, 3000), rng.uniform(3000, 9000)))
            else:
                rx.append("  SRI / %.4f %.2f %.2f /" % (rng.uniform(0.5, 2.0), rng.uniform(100, 3000),
                                                      rng.uniform(200, 3000)))
            effs = rng.choice(len(comps), size=2, replace=False)
            rx.append("  " + " ".join("%s/%.2f/" % (_name(comps[e]), rng.uniform(0.5, 5.0)) for e in effs))
        elif kind == "plog":
            rx.append("%s <=> %s  %s %.4f %.3f" % (lhs, rhs, _fmt(A), b, Ea))
            for p in (0.1, 1.0, 10.0, 100.0):
                rx.append("  PLOG / %.3f %s %.4f %.3f /" % (
                    p, _fmt(A * float(np.exp(rng.uniform(-2, 2)))), b + float(rng.uniform(-0.5, 0.5)),
                    Ea * float(rng.uniform(0.8, 1.2))))
        elif kind == "cheb":
            rx.append("%s (+M) <=> %s (+M)  1.0 0.0 0.0" % (lhs, rhs))
            rx.append("  TCHEB / 300.0 3000.0 /  PCHEB / 0.01 100.0 /")
            coeffs = rng.normal(0.0, 0.3, size=(6, 4))
            coeffs[0, 0] = np.log10(A) + (order - 1) * 3.0 * 0 + 0.0
            coeffs[0, 0] = float(rng.uniform(8.0, 13.0))
            rx.append("  CHEB / 6 4 /")
            flat = coeffs.ravel()
            for k in range(0, len(flat), 4):
                rx.append("  CHEB / " + " ".join("%.5E" % x for x in flat[k:k + 4]) + " /")
        made += 1
    if made < n_reactions:
        raise RuntimeError("could not generate %d reactions" % n_reactions)
    rx.append("END")
    return body + "\n".join(rx) + "\n"


def write(path, **kw):
    text = generate(**kw)
    with open(path, "w") as fh:
        fh.write(text)
    return path

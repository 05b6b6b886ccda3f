"""Chemkin-II mechanism and NASA-7 thermo reader.

Produces the same species list, reaction list, parameters (after unit
conversion) and reaction classification as pyJac's ``read_mech``
(pyjac/core/mech_interpret.py:106-809) and ``read_thermo`` (:812-969), so
that every table derived from it is bit-identical to the reference's:

* sections ELEMENTS / SPECIES / REACTIONS / THERMO / END, ``!`` comments;
* REACTIONS-line units (pre-exponential ``moles``; activation energy in
  cal/mole, kcal/mole, joules/mole, kjoules/mole, joules/kmole, kelvins,
  evolts), converted exactly as the reference does (:450-466, :549-567);
* ``<=>``, ``=>``, ``=``; ``+ M`` third bodies; ``(+M)`` / ``(+SPECIES)``
  fall-off; auxiliary DUP, REV, LOW, HIGH, TROE (zero T*** / T* replaced by
  1e-30, :618-629), SRI, CHEB/PCHEB/TCHEB, PLOG and efficiency lines;
* reactions with explicit REV parameters split into two irreversible
  reactions (:759-775);
* classification into elementary / thd / fall / chem / plog / cheb,
  third-body kind (none / mix / unity / species) and fall-off form
  (none / lind / troe / sri) as ``ReacInfo.finalize`` (chem_model.py:275-339).

Thermo entries are NASA-7 polynomials in fixed columns (name 0:18, element
counts 24:44 in 5-column groups, temperatures 45:74, four lines per species).
"""
import copy
import math

from .elements import (ACT_ENERGY_FACTOR, PA, PRE_UNITS, atomic_weights)

# reaction kinds (values follow pyjac/core/enum_types.py reaction_type)
ELEMENTARY, THD, FALL, CHEM, PLOG, CHEB = 1, 2, 3, 4, 5, 6
# third-body kinds (enum_types.thd_body_type)
THD_NONE, THD_MIX, THD_SPECIES, THD_UNITY = 0, 1, 2, 3
# fall-off blending (enum_types.falloff_form)
FALL_NONE, FALL_LIND, FALL_TROE, FALL_SRI = 0, 1, 2, 3


class ChemkinError(ValueError):
    """Malformed or unsupported mechanism input."""


class Species(object):
    def __init__(self, name):
        self.name = name
        self.elem = []           # [[element, count], ...]
        self.mw = 0.0            # kg / kmol
        self.hi = [0.0] * 7      # NASA-7 high-temperature coefficients
        self.lo = [0.0] * 7      # NASA-7 low-temperature coefficients
        self.Trange = [300.0, 1000.0, 5000.0]

    def __repr__(self):
        return "Species(%s)" % self.name


class Reaction(object):
    def __init__(self, rev, reac, reac_nu, prod, prod_nu, A, b, E):
        self.reac, self.reac_nu = list(reac), list(reac_nu)
        self.prod, self.prod_nu = list(prod), list(prod_nu)
        self.A, self.b, self.E = A, b, E        # SI-kmol units, E in Kelvin
        self.rev = rev
        self.rev_par = []
        self.dup = False
        self.thd_body = False
        self.thd_body_eff = []                  # [[species, efficiency], ...]
        self.pdep = False
        self.pdep_sp = ''
        self.low = []
        self.high = []
        self.troe = False
        self.troe_par = []
        self.sri = False
        self.sri_par = []
        self.cheb = False
        self.cheb_n_temp = 0
        self.cheb_n_pres = 0
        self.cheb_plim = [0.001 * PA, 100. * PA]
        self.cheb_tlim = [300., 2500.]
        self.cheb_par = None
        self.plog = False
        self.plog_par = None
        # classification (set by finalize)
        self.kind = None
        self.thd_kind = THD_NONE
        self.fall_form = FALL_NONE
        self.rxn_str = ''

    # -- classification, pyjac/core/chem_model.py:275-380 -------------------
    def finalize(self, num_species):
        if self.thd_body:
            self.kind = THD
        elif self.pdep and self.low:
            self.kind = FALL
        elif self.pdep and self.high:
            self.kind = CHEM
        elif self.plog:
            self.kind = PLOG
        elif self.cheb:
            self.kind = CHEB
        else:
            self.kind = ELEMENTARY
        if self.kind in (FALL, CHEM, THD):
            if self.pdep_sp:
                self.thd_kind = THD_SPECIES
            elif not self.thd_body_eff or (len(self.thd_body_eff) == num_species and
                                           all(t[1] == 1.0 for t in self.thd_body_eff)):
                self.thd_kind = THD_UNITY
            else:
                self.thd_kind = THD_MIX
        else:
            self.thd_kind = THD_NONE
        if self.kind in (FALL, CHEM):
            self.fall_form = FALL_TROE if self.troe else (FALL_SRI if self.sri else FALL_LIND)
        else:
            self.fall_form = FALL_NONE
        if self.plog or self.cheb:
            self.A = 0
            self.b = 0
            self.E = 0
        self.rxn_str = self._describe()

    def _side(self, species, nus):
        out = []
        for s, nu in zip(species, nus):
            nu_str = str(int(nu)) if float(nu).is_integer() else str(nu)
            out.append(s if nu == 1 else "%s %s" % (nu_str, s))
        txt = " + ".join(out)
        if self.kind in (FALL, CHEM):
            txt += " (+%s)" % self.pdep_sp if self.pdep_sp else " (+M)"
        elif self.kind == THD:
            txt += " + M"
        return txt

    def _describe(self):
        head = {FALL: "FalloffReaction: ", CHEM: "ChemicallyActivatedReaction: ",
                THD: "ThreeBodyReaction: ", PLOG: "PLOGReaction: ",
                CHEB: "ChebyshevReaction: "}.get(self.kind, "ElementaryReaction: ")
        arrow = " <=> " if self.rev else " => "
        return head + self._side(self.reac, self.reac_nu) + arrow + \
            self._side(self.prod, self.prod_nu)

    def __repr__(self):
        return self.rxn_str or "Reaction(unfinalized)"


def _strip_comment(line):
    line = line.strip()
    ind = line.find('!')
    if ind > 0:
        line = line[:ind]
    return line


def _blank_or_comment(line):
    s = line.strip()
    return (not s) or s.startswith('!')


def _split_side(text):
    """Split one side of a reaction equation; return (species, nus, thd, pdep, pdep_sp)."""
    thd = pdep = False
    pdep_sp = ''
    sub = text
    # look for a '(+M)' / '(+SPECIES)' group that is not part of a species name
    while '(' in sub:
        i1 = sub.find('(')
        i2 = sub.find(')')
        inner = sub[i1 + 1:i2].strip()
        if inner == '+':
            sub = sub[i2 + 1:]
        elif inner[:1] == '+':
            pdep = True
            pdep_sp = sub[i1 + 1:i2].replace('+', ' ').strip()
            if pdep_sp.lower() == 'm':
                thd = True
                pdep_sp = ''
            base = text.find(sub)
            text = text[:i1 + base] + text[i2 + base + 1:]
            break
        else:
            sub = sub[i2 + 1:]
    parts = text.split('+')
    # consecutive '+' means the species name itself ended in '+'
    while '' in parts:
        k = parts.index('')
        parts[k - 1] = parts[k - 1] + '+'
        del parts[k]
    # re-join species such as 'A(+)B' that the split above broke apart
    for sp in list(parts):
        k = parts.index(sp)
        if k < len(parts) - 1:
            nxt = parts[k + 1]
            if sp[-1:] == '(' and nxt[:1] == ')':
                parts[k] = sp + '+' + nxt
                del parts[k + 1]
    names, nus = [], []
    for sp in parts:
        sp = sp.strip()
        if sp[:1].isdigit():
            i = 0
            for i in range(len(sp)):
                if sp[i:i + 1].isalpha():
                    break
            num = sp[:i]
            nu = float(num) if '.' in num else int(num)
            sp = sp[i:].strip()
        else:
            nu = 1
        if sp in ('m', 'M'):
            thd = True
            continue
        if sp not in names:
            names.append(sp)
            nus.append(nu)
        else:
            nus[names.index(sp)] += nu
    return names, nus, thd, pdep, pdep_sp


def _floats_after_keyword(line):
    return line.replace('/', ' ').replace(',', ' ').split()


def read_mech(mech_filename, therm_filename=None):
    """Parse a Chemkin mechanism; return (elements, species, reactions)."""
    wt = atomic_weights()
    elems, specs, reacs = [], [], []
    key = ''
    units_E, units_A = 'cal/mole', 'moles'
    thd = pdep = False
    cheb_flag = False
    with open(mech_filename, 'r') as fh:
        lines = fh.readlines()
    for raw in lines:
        if _blank_or_comment(raw):
            continue
        line = _strip_comment(raw)
        head = line[:4].lower()
        if head == 'elem' or head == 'spec':
            key = head
            toks = line.split()
            if len(toks) > 1:
                line = line[line.index(toks[1]):]
            else:
                continue
        elif head == 'reac':
            key = 'reac'
            units_E, units_A = 'cal/mole', 'moles'
            for unit in line.split()[1:]:
                u = unit.lower()
                if u in PRE_UNITS:
                    units_A = u
                elif u in ACT_ENERGY_FACTOR:
                    units_E = u
                else:
                    raise ChemkinError("unsupported units on REACTION line: %s" % unit)
            if units_A == 'molecules':
                raise NotImplementedError("molecules units are not supported")
            continue
        elif head == 'ther':
            _read_thermo(mech_filename, specs, wt)
            continue
        elif line[:3].lower() == 'end':
            key = ''
            continue

        if key == 'elem':
            last = ''
            for e in line.replace('/', ' ').split():
                if e.isalpha():
                    if e[:3] == 'end':
                        continue
                    if e not in elems:
                        elems.append(e)
                    last = e
                else:
                    wt[last.lower()] = float(e)
        elif key == 'spec':
            for s in line.split():
                if s[:3] == 'end':
                    continue
                if not any(sp.name == s for sp in specs):
                    specs.append(Species(s))
        elif key == 'reac':
            if '=' in line:
                cheb_flag = False
                toks = line.split()
                n = len(toks)
                A, b, E = float(toks[n - 3]), float(toks[n - 2]), float(toks[n - 1])
                eq = line[:line.index(toks[n - 3])].strip()
                if '<=>' in eq:
                    i = eq.index('<=>')
                    rev, lhs, rhs = True, eq[:i].strip(), eq[i + 3:].strip()
                elif '=>' in eq:
                    i = eq.index('=>')
                    rev, lhs, rhs = False, eq[:i].strip(), eq[i + 2:].strip()
                else:
                    i = eq.index('=')
                    rev, lhs, rhs = True, eq[:i].strip(), eq[i + 1:].strip()
                rs, rnu, thd_l, pdep_l, psp_l = _split_side(lhs)
                ps, pnu, thd_r, pdep_r, psp_r = _split_side(rhs)
                thd = thd_l or thd_r
                pdep = pdep_l or pdep_r
                pdep_sp = psp_r if pdep_r else psp_l
                if pdep:
                    thd = False
                E *= ACT_ENERGY_FACTOR[units_E]
                if units_A == 'moles':
                    order = sum(rnu)
                    if thd:
                        A /= 1000. ** order
                    else:
                        A /= 1000. ** (order - 1.)
                r = Reaction(rev, rs, rnu, ps, pnu, A, b, E)
                r.thd_body = thd
                r.pdep = pdep
                if pdep:
                    r.pdep_sp = pdep_sp
                reacs.append(r)
            else:
                _aux(line, reacs, units_A, units_E, thd, pdep, cheb_flag)
                if line[:3].lower() == 'che':
                    cheb_flag = True

    for idx, r in enumerate(reacs):
        if r.cheb:
            nT, nP = r.cheb_n_temp, r.cheb_n_pres
            if len(r.cheb_par) != nT * nP:
                raise ChemkinError("incorrect number of CHEB coefficients in reaction %d" % idx)
            if units_A == 'moles':
                r.cheb_par[0] += math.log10(0.001 ** (sum(r.reac_nu) - 1.))
            r.cheb_par = [r.cheb_par[i * nP:(i + 1) * nP] for i in range(nT)]

    names = set(s.name for s in specs)
    for idx, r in enumerate(reacs):
        for s in r.reac + r.prod:
            if s not in names:
                raise ChemkinError("reaction %d contains unknown species %s" % (idx, s))

    # explicit reverse parameters -> two irreversible reactions
    for r in list(reacs):
        if r.rev_par:
            back = copy.deepcopy(r)
            k = reacs.index(r)
            r.rev = False
            r.rev_par = []
            back.A, back.b, back.E = back.rev_par[0], back.rev_par[1], back.rev_par[2]
            back.rev = False
            back.rev_par = []
            back.prod, back.prod_nu = r.reac[:], r.reac_nu[:]
            back.reac, back.reac_nu = r.prod[:], r.prod_nu[:]
            reacs.insert(k + 1, back)

    if any(not s.mw for s in specs):
        if therm_filename:
            _read_thermo(therm_filename, specs, wt)
        else:
            raise ChemkinError("no thermo file given and the mechanism lacks thermo data")
    missing = [s.name for s in specs if not s.mw]
    if missing:
        raise ChemkinError("missing thermo data for " + ", ".join(missing))

    for r in reacs:
        r.finalize(len(specs))
    for s in specs:
        s.elem = [e for e in s.elem if e[1] != 0]
    return elems, specs, reacs


def _aux(line, reacs, units_A, units_E, thd, pdep, cheb_flag):
    """Auxiliary reaction line (pyjac/core/mech_interpret.py:525-735)."""
    r = reacs[-1]
    aux = line[:3].lower()
    if aux == 'dup':
        r.dup = True
    elif aux == 'rev':
        t = _floats_after_keyword(line)
        p1, p2, p3 = float(t[1]), float(t[2]), float(t[3])
        p3 *= ACT_ENERGY_FACTOR[units_E]
        if units_A == 'moles':
            order = sum(r.prod_nu)
            if thd:
                p1 /= 1000. ** order
            else:
                p1 /= 1000. ** (order - 1.)
        if p1 != 0.0:
            r.rev_par.extend([p1, p2, p3])
        else:
            r.rev = False
    elif aux == 'low':
        t = _floats_after_keyword(line)
        p1, p2, p3 = float(t[1]), float(t[2]), float(t[3])
        p3 *= ACT_ENERGY_FACTOR[units_E]
        if units_A == 'moles':
            p1 /= 1000. ** sum(r.reac_nu)
        r.low.extend([p1, p2, p3])
    elif aux == 'hig':
        t = _floats_after_keyword(line)
        p1, p2, p3 = float(t[1]), float(t[2]), float(t[3])
        p3 *= ACT_ENERGY_FACTOR[units_E]
        if units_A == 'moles':
            p1 /= 1000. ** (sum(r.reac_nu) - 2.)
        r.high.extend([p1, p2, p3])
    elif aux == 'tro':
        t = _floats_after_keyword(line)
        r.troe = True
        p1, p2, p3 = float(t[1]), float(t[2]), float(t[3])
        p2 = 1e-30 if p2 == 0 else p2
        p3 = 1e-30 if p3 == 0 else p3
        r.troe_par.extend([p1, p2, p3])
        if len(t) > 4:
            r.troe_par.append(float(t[4]))
    elif aux == 'sri':
        t = _floats_after_keyword(line)
        r.sri = True
        r.sri_par.extend([float(t[1]), float(t[2]), float(t[3])])
        if len(t) > 4:
            r.sri_par.extend([float(t[4]), float(t[5])])
    elif aux == 'che':
        r.cheb = True
        t = line.replace('/', ' ').split()
        if cheb_flag:
            r.cheb_par.extend(float(x) for x in t[1:])
        else:
            r.pdep = False
            r.cheb_n_temp = int(t[1])
            r.cheb_n_pres = int(t[2])
            r.cheb_par = [float(x) for x in t[3:]]
    elif aux == 'pch':
        t = line.replace('/', ' ').split()
        r.cheb_plim = [float(t[1]) * PA, float(t[2]) * PA]
        if len(t) > 3 and t[3].lower() == 'tcheb':
            r.cheb_tlim = [float(t[4]), float(t[5])]
    elif aux == 'tch':
        t = line.replace('/', ' ').split()
        r.cheb_tlim = [float(t[1]), float(t[2])]
        if len(t) > 3 and t[3].lower() == 'pcheb':
            r.cheb_plim = [float(t[4]) * PA, float(t[5]) * PA]
    elif aux == 'plo':
        t = line.replace('/', ' ').split()
        if not r.plog:
            r.plog = True
            r.pdep = False
            r.plog_par = []
        pars = [float(x) for x in t[1:5]]
        pars[0] *= 101325.0
        pars[3] *= ACT_ENERGY_FACTOR[units_E]
        if units_A == 'moles':
            pars[1] /= 1000. ** (sum(r.reac_nu) - 1.)
        r.plog_par.append(pars)
    else:
        t = line.replace('/', ' ').split()
        for i in range(0, len(t), 2):
            r.thd_body_eff.append([t[i], float(t[i + 1])])


def _split_fixed(s, width):
    return [s[i:i + width] for i in range(0, len(s), width)]


def _read_thermo(filename, specs, wt):
    """NASA-7 thermo reader (pyjac/core/mech_interpret.py:812-969)."""
    T_common = None
    with open(filename, 'r') as fh:
        lines = fh.readlines()
    i = 0
    n = len(lines)
    while i < n:
        line = lines[i]
        i += 1
        if _blank_or_comment(line):
            continue
        if 'thermo' in line.lower():
            break
    if i < n:
        toks = lines[i].split()
        if toks and toks[0][:1].isdigit():
            T_common = [float(x) for x in lines[i].split()]
            i += 1
    by_name = {s.name: s for s in specs}
    while i < n:
        line = lines[i]
        i += 1
        if line[:3].lower() == 'end':
            break
        if _blank_or_comment(line):
            continue
        name = line[0:18].strip()
        if name.find(' ') > 0:
            name = name[:name.find(' ')]
        sp = by_name.get(name)
        if sp is None or sp.mw:
            i += 3
            continue
        for grp in _split_fixed(line[24:44], 5):
            e = grp[0:2].strip()
            if e == '' or e == '0':
                continue
            cnt = int(float(grp[2:].strip()))
            sp.elem.append([e, cnt])
            sp.mw += cnt * wt[e.lower()]
        Ts = [float(x) for x in line[45:74].split()]
        T_com = Ts[2] if len(Ts) == 3 else (T_common[1] if T_common else 1000.0)
        sp.Trange = [Ts[0], T_com, Ts[1]]
        l2, l3, l4 = lines[i], lines[i + 1], lines[i + 2]
        i += 3
        c2 = _split_fixed(l2[0:75], 15)
        c3 = _split_fixed(l3[0:75], 15)
        c4 = _split_fixed(l4[0:75], 15)
        sp.hi = [float(c2[0]), float(c2[1]), float(c2[2]), float(c2[3]), float(c2[4]),
                 float(c3[0]), float(c3[1])]
        sp.lo = [float(c3[2]), float(c3[3]), float(c3[4]),
                 float(c4[0]), float(c4[1]), float(c4[2]), float(c4[3])]
        if not any(s.mw == 0.0 for s in specs):
            break

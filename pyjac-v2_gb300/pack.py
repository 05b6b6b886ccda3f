"""Pack a Mechanism's tables into the device layout of csrc/pjg_tables.cuh.

Input is the reference-layout table dictionary (``Mechanism.val``, the same
fields as pyjac/core/rate_subs.py:assign_rates and
create_jacobian.py:determine_jac_inds); output is a set of numpy arrays whose
bytes are handed to ``pjg_mech_create`` through the ``pjg_tables`` struct.
"""
import numpy as np

from .mech.elements import PA, RU

MAXSP = 8
RXN_BYTES = 192

FORM_A, FORM_AT, FORM_ARR, FORM_PLOG, FORM_CHEB = 0, 1, 2, 3, 4
RX_REV = 1 << 3
RX_THD_SHIFT = 4
RX_BLEND_SHIFT = 6
RX_CHEM = 1 << 8
RX_FFORM_SHIFT = 9
RX_HASNS = 1 << 11
RX_NSLIST = 1 << 12
RX_T2 = 1 << 13
RX_SRID = 1 << 14
RX_SRIE = 1 << 15
RX_SRIEINT = 1 << 16

P_A, P_B, P_TA, P_FA, P_FB, P_FTA = 0, 1, 2, 3, 4, 5
P_F0, P_F1, P_F2, P_F3, P_F4 = 6, 7, 8, 9, 10
P_PSUM, P_FLAG, P_CNS, P_MOD = 11, 12, 13, 14

RXN_DTYPE = np.dtype([("flags", "<i4"), ("nspec", "<i4"), ("thd_off", "<i4"), ("thd_cnt", "<i4"),
                      ("aux", "<i4"), ("nu_sum", "<i4"), ("bint", "<i4"), ("fbint", "<i4"),
                      ("ent", "<u4", (MAXSP,)), ("p", "<f8", (16,))])
assert RXN_DTYPE.itemsize == RXN_BYTES


def _powi(v, p):
    """The reference's fast_powi (repeated multiplication, left to right)."""
    if p < 0:
        v = 1.0 / v
        p = -p
    if p == 0:
        return 1.0
    r = v
    for _ in range(p - 1):
        r = r * v
    return r


def _offsets(counts):
    return np.concatenate(([0], np.cumsum(np.asarray(counts, dtype=np.int64)))).astype(np.int64)


def _form(t):
    t = int(t)
    return t if t <= 1 else FORM_ARR


class PackedTables(object):
    """Device-layout arrays for one mechanism (kept alive while in use)."""

    def __init__(self, mech):
        v = mech.val
        Ns, Nr = int(v["Ns"]), int(v["Nr"])
        last = Ns - 1
        self.ns, self.nr = Ns, Nr
        rx = np.zeros(Nr, dtype=RXN_DTYPE)

        def inv(mp):
            out = -np.ones(Nr, dtype=np.int64)
            out[np.asarray(mp, dtype=np.int64)] = np.arange(len(mp))
            return out

        r_simple = inv(v["simple"]["map"])
        r_plog = inv(v["plog"]["map"])
        r_cheb = inv(v["cheb"]["map"])
        r_thd = inv(v["thd"]["map"])
        r_fall = inv(v["fall"]["map"])
        rev = set(int(x) for x in v["rev"]["map"])
        net_off = _offsets(v["net"]["num_reac_to_spec"])
        net_spec = np.asarray(v["net"]["reac_to_spec"])
        net_nu = np.asarray(v["net"]["nu"])
        thd_off = _offsets(v["thd"]["spec_num"])
        fall = v["fall"]
        troe_of = inv_fall(fall["troe"]["map"], int(fall["num"]))
        sri_of = inv_fall(fall["sri"]["map"], int(fall["num"]))

        thd_spec, thd_coef, aux = [], [], []
        need_logP = False
        for i in range(Nr):
            rec = rx[i]
            p = np.zeros(16)
            flags = 0
            o0, o1 = int(net_off[i]), int(net_off[i + 1])
            nsp = o1 - o0
            if nsp > MAXSP:
                raise ValueError("reaction %d has %d species; the kernels support %d"
                                 % (i, nsp, MAXSP))
            ents = []
            has_ns = False
            for e in range(o0, o1):
                sp = int(net_spec[e])
                nur, nuf = int(net_nu[2 * e]), int(net_nu[2 * e + 1])
                if not (0 <= nuf < 256 and 0 <= nur < 256):
                    raise ValueError("stoichiometric coefficient out of range in reaction %d" % i)
                ents.append(sp | (nuf << 16) | (nur << 24))
                has_ns |= sp == last
            rec["ent"][:nsp] = ents
            rec["nspec"] = nsp
            rec["nu_sum"] = int(v["net"]["nu_sum"][i])
            if has_ns:
                flags |= RX_HASNS
            si = r_simple[i]
            if si >= 0:
                form = _form(v["simple"]["type"][si])
                p[P_A] = v["simple"]["A"][si]
                p[P_B] = v["simple"]["b"][si]
                p[P_TA] = v["simple"]["Ta"][si]
                if form == FORM_AT:
                    rec["bint"] = int(p[P_B])
            elif r_plog[i] >= 0:
                form = FORM_PLOG
                need_logP = True
                pi = r_plog[i]
                nP = int(v["plog"]["num_P"][pi])
                pp = v["plog"]["post_process"]["params"]
                rec["aux"] = len(aux)
                aux.append(float(nP))
                for j in range(nP):
                    aux.extend(float(pp[m, pi, j]) for m in range(4))
            else:
                form = FORM_CHEB
                need_logP = True
                ci = r_cheb[i]
                ch = v["cheb"]
                nT, nP = int(ch["num_T"][ci]), int(ch["num_P"][ci])
                tl = ch["post_process"]["Tlim"][ci]
                pl = ch["post_process"]["Plim"][ci]
                rec["aux"] = len(aux)
                aux.extend([float(nT), float(nP), float(tl[0]), float(tl[1]), float(pl[0]),
                            float(pl[1])])
                aux.extend(np.asarray(ch["post_process"]["params"][ci][:nT, :nP],
                                      dtype=np.float64).ravel().tolist())
            flags |= form
            if i in rev:
                flags |= RX_REV
                nu = int(v["net"]["nu_sum"][i])
                pval = PA / RU if nu > 0 else RU / PA
                p[P_PSUM] = 1.0 / _powi(pval, abs(nu))
            ti = r_thd[i]
            if ti >= 0:
                ttype = int(v["thd"]["type"][ti])      # 1 mix, 2 species, 3 unity
                flags |= ttype << RX_THD_SHIFT
                flag = 0.0 if ttype == 2 else 1.0
                p[P_FLAG] = flag
                rec["thd_off"] = len(thd_spec)
                cns = 0.0
                for e in range(int(thd_off[ti]), int(thd_off[ti + 1])):
                    sp = int(v["thd"]["spec"][e])
                    coef = float(v["thd"]["eff"][e]) - flag
                    thd_spec.append(sp)
                    thd_coef.append(coef)
                    if sp == last:
                        flags |= RX_NSLIST
                        cns = coef
                rec["thd_cnt"] = int(thd_off[ti + 1] - thd_off[ti])
                p[P_CNS] = cns
                p[P_MOD] = flag + cns
            fi = r_fall[i]
            if fi >= 0:
                blend = int(fall["blend"][fi])
                flags |= blend << RX_BLEND_SHIFT
                if int(fall["ftype"][fi]):
                    flags |= RX_CHEM
                fform = _form(fall["type"][fi])
                flags |= fform << RX_FFORM_SHIFT
                p[P_FA] = fall["A"][fi]
                p[P_FB] = fall["b"][fi]
                p[P_FTA] = fall["Ta"][fi]
                if fform == FORM_AT:
                    rec["fbint"] = int(p[P_FB])
                if troe_of[fi] >= 0:
                    q = troe_of[fi]
                    tr = fall["troe"]
                    p[P_F0], p[P_F1], p[P_F2], p[P_F3] = tr["a"][q], tr["T1"][q], tr["T2"][q], tr["T3"][q]
                    if tr["T2"][q] != 0.0:
                        flags |= RX_T2
                elif sri_of[fi] >= 0:
                    q = sri_of[fi]
                    sr = fall["sri"]
                    p[P_F0], p[P_F1], p[P_F2] = sr["a"][q], sr["b"][q], sr["c"][q]
                    p[P_F3], p[P_F4] = sr["d"][q], sr["e"][q]
                    if sr["d"][q] != 1.0:
                        flags |= RX_SRID
                    if sr["e"][q] != 0.0:
                        flags |= RX_SRIE
                        if float(sr["e"][q]).is_integer():
                            flags |= RX_SRIEINT
            rec["flags"] = flags
            rec["p"] = p
        self.rxn = rx
        self.species = species_records(v)
        self.thd_spec = np.asarray(thd_spec if thd_spec else [0], dtype=np.int32)
        self.thd_coef = np.asarray(thd_coef if thd_coef else [0.0], dtype=np.float64)
        self.n_thd = len(thd_spec)
        self.aux = np.asarray(aux if aux else [0.0], dtype=np.float64)
        self.n_aux = len(aux)
        # bit 0: PLOG / Chebyshev present (ln P needed); bit 1: the 'approximate'
        # Jacobian type (no bath-gas terms in the species columns)
        self.flags = (1 if need_logP else 0) | (2 if getattr(mech, "jac_type", "exact") == "approximate" else 0)
        ji = v["jac_inds"]
        self.crs_row_ptr = np.ascontiguousarray(ji["crs"]["row_ptr"], dtype=np.int32)
        self.crs_col_ind = np.ascontiguousarray(ji["crs"]["col_ind"], dtype=np.int32)
        self.ccs_col_ptr = np.ascontiguousarray(ji["ccs"]["col_ptr"], dtype=np.int32)
        self.ccs_row_ind = np.ascontiguousarray(ji["ccs"]["row_ind"], dtype=np.int32)
        self.nnz = int(self.crs_col_ind.size)


SP_DOUBLES, SP_LO, SP_HI = 48, 8, 28


def species_records(v):
    """Species records of csrc/pjg_tables.cuh: T_mid, W_k/W_ns, 1 - W_k/W_ns and,
    per temperature range, the NASA-7 coefficients with the polynomial quotients
    of rate_subs.py:3335-3356 formed once here."""
    Ns = int(v["Ns"])
    th = v["thermo"]
    sp = np.zeros((Ns, SP_DOUBLES))
    sp[:, 0] = th["T_mid"]
    sp[:Ns - 1, 1] = v["mw_post"]
    sp[:, 2] = 1.0 - sp[:, 1]
    sp[Ns - 1, 2] = 0.0
    for base, a in ((SP_LO, th["a_lo"]), (SP_HI, th["a_hi"])):
        a = np.asarray(a, dtype=np.float64)
        sp[:, base:base + 7] = a
        sp[:, base + 7] = a[:, 1] / 2.0
        sp[:, base + 8] = a[:, 2] / 3.0
        sp[:, base + 9] = a[:, 3] / 4.0
        sp[:, base + 10] = a[:, 4] / 5.0
        sp[:, base + 11] = a[:, 1] / 2.0
        sp[:, base + 12] = a[:, 2] / 6.0
        sp[:, base + 13] = a[:, 3] / 12.0
        sp[:, base + 14] = a[:, 4] / 20.0
        sp[:, base + 15] = 2.0 * a[:, 2]
        sp[:, base + 16] = 3.0 * a[:, 3]
        sp[:, base + 17] = 4.0 * a[:, 4]
        sp[:, base + 18] = a[:, 0] - 1.0
        sp[:, base + 19] = a[:, 6] - a[:, 0]
    return np.ascontiguousarray(sp)


def inv_fall(mp, n):
    out = -np.ones(max(n, 1), dtype=np.int64)
    out[np.asarray(mp, dtype=np.int64)] = np.arange(len(mp))
    return out

"""Python side of the CPU oracle (test infrastructure only).

Builds ``oracle/pyjac_oracle.c`` into ``oracle/_build/liboracle.so`` with gcc
and exposes :class:`Oracle`, which evaluates species rates and the dense
analytical Jacobian of a mechanism on the CPU from the reference-layout tables
(``Mechanism.val``).  Also wraps the shim-compiled reference kernels in
``oracle/_ref`` (:class:`RefKernels`) when they were built in this tree.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use this module, and only as the checker / the timed CPU
baseline.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRC = os.path.join(HERE, "pyjac_oracle.c")
HDR = os.path.join(HERE, "pyjac_oracle.h")
COUNT_SRC = os.path.join(HERE, "flop_count.cpp")
COUNT_LIB = os.path.join(BUILD, "liboracle_count.so")


def build(force=False, quiet=True):
    os.makedirs(BUILD, exist_ok=True)
    if (not force and os.path.exists(LIB) and
            os.path.getmtime(LIB) >= max(os.path.getmtime(SRC), os.path.getmtime(HDR))):
        return LIB
    cmd = ["gcc", "-O2", "-std=c99", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           SRC, "-o", LIB + ".tmp", "-lm"]
    if not quiet:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def build_counter(force=False, quiet=True):
    """The operation-counting build of the same oracle source (flop_count.cpp)."""
    os.makedirs(BUILD, exist_ok=True)
    deps = [SRC, HDR, COUNT_SRC]
    if (not force and os.path.exists(COUNT_LIB) and
            os.path.getmtime(COUNT_LIB) >= max(os.path.getmtime(d) for d in deps)):
        return COUNT_LIB
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-w", "-ffp-contract=off", "-I", HERE,
           COUNT_SRC, "-o", COUNT_LIB + ".tmp", "-lm"]
    if not quiet:
        print(" ".join(cmd))
    subprocess.check_call(cmd)
    os.replace(COUNT_LIB + ".tmp", COUNT_LIB)
    return COUNT_LIB


OP_NAMES = ("add", "mul", "div", "fma", "minmax", "exp", "log", "log10", "pow", "sqrt")


_I = ctypes.POINTER(ctypes.c_int)
_D = ctypes.POINTER(ctypes.c_double)


class _OrcMech(ctypes.Structure):
    _fields_ = [("ns", ctypes.c_int), ("nr", ctypes.c_int),
                ("net_off", _I), ("net_spec", _I), ("net_nu", _I), ("nu_sum", _I),
                ("rev_mask", _I),
                ("rxn_simple", _I), ("rxn_plog", _I), ("rxn_cheb", _I), ("rxn_thd", _I),
                ("rxn_fall", _I),
                ("simple_type", _I), ("simple_A", _D), ("simple_b", _D), ("simple_Ta", _D),
                ("plog_maxP", ctypes.c_int), ("plog_numP", _I), ("plog_params", _D),
                ("n_plog", ctypes.c_int),
                ("cheb_maxT", ctypes.c_int), ("cheb_maxP", ctypes.c_int), ("n_cheb", ctypes.c_int),
                ("cheb_nT", _I), ("cheb_nP", _I), ("cheb_params", _D), ("cheb_Plim", _D),
                ("cheb_Tlim", _D),
                ("thd_type", _I), ("thd_off", _I), ("thd_spec", _I), ("thd_eff", _D),
                ("fall_ftype", _I), ("fall_blend", _I), ("fall_type", _I),
                ("fall_A", _D), ("fall_b", _D), ("fall_Ta", _D),
                ("fall_troe", _I), ("fall_sri", _I),
                ("troe_a", _D), ("troe_T1", _D), ("troe_T2", _D), ("troe_T3", _D),
                ("sri_a", _D), ("sri_b", _D), ("sri_c", _D), ("sri_d", _D), ("sri_e", _D),
                ("a_lo", _D), ("a_hi", _D), ("T_mid", _D), ("mw_post", _D),
                ("jac_approx", ctypes.c_int)]


def _offsets(counts):
    counts = np.asarray(counts, dtype=np.int64)
    return np.concatenate(([0], np.cumsum(counts))).astype(np.int32)


class Oracle(object):
    """CPU evaluation of species rates and the dense Jacobian (C order in/out)."""

    def __init__(self, mech):
        self._lib = ctypes.CDLL(build())
        for fn in (self._lib.orc_species_rates, self._lib.orc_jacobian, self._lib.orc_rates_scale):
            fn.restype = ctypes.c_int
            fn.argtypes = [ctypes.POINTER(_OrcMech), ctypes.c_long, ctypes.c_int, _D, _D, _D,
                           ctypes.c_int]
        self._lib.orc_chem_utils.restype = ctypes.c_int
        self._lib.orc_chem_utils.argtypes = [ctypes.POINTER(_OrcMech), ctypes.c_long, ctypes.c_int,
                                             _D, _D, _D, _D]
        self.mech = mech
        v = mech.val
        Ns, Nr = v["Ns"], v["Nr"]
        keep = self._keep = []

        def I(a):
            a = np.ascontiguousarray(np.asarray(a, dtype=np.int32).ravel())
            if a.size == 0:
                a = np.zeros(1, dtype=np.int32)
            keep.append(a)
            return a.ctypes.data_as(_I)

        def D(a):
            a = np.ascontiguousarray(np.asarray(a, dtype=np.float64).ravel())
            if a.size == 0:
                a = np.zeros(1)
            keep.append(a)
            return a.ctypes.data_as(_D)

        def rxn_index(mp):
            out = -np.ones(Nr, dtype=np.int32)
            out[np.asarray(mp, dtype=np.int64)] = np.arange(len(mp))
            return out

        fall = v["fall"]
        nfall = int(fall["num"])
        fall_troe = -np.ones(max(nfall, 1), dtype=np.int32)
        fall_troe[np.asarray(fall["troe"]["map"], dtype=np.int64)] = np.arange(fall["troe"]["num"])
        fall_sri = -np.ones(max(nfall, 1), dtype=np.int32)
        fall_sri[np.asarray(fall["sri"]["map"], dtype=np.int64)] = np.arange(fall["sri"]["num"])
        rev_mask = rxn_index(v["rev"]["map"])
        plog = v["plog"]
        cheb = v["cheb"]
        m = _OrcMech()
        m.ns, m.nr = Ns, Nr
        m.net_off = I(_offsets(v["net"]["num_reac_to_spec"]))
        m.net_spec = I(v["net"]["reac_to_spec"])
        m.net_nu = I(v["net"]["nu"])
        m.nu_sum = I(v["net"]["nu_sum"])
        m.rev_mask = I(rev_mask)
        m.rxn_simple = I(rxn_index(v["simple"]["map"]))
        m.rxn_plog = I(rxn_index(plog["map"]))
        m.rxn_cheb = I(rxn_index(cheb["map"]))
        m.rxn_thd = I(rxn_index(v["thd"]["map"]))
        m.rxn_fall = I(rxn_index(fall["map"]))
        m.simple_type = I(v["simple"]["type"])
        m.simple_A = D(v["simple"]["A"])
        m.simple_b = D(v["simple"]["b"])
        m.simple_Ta = D(v["simple"]["Ta"])
        m.n_plog = int(plog["num"])
        m.plog_maxP = int(plog["max_P"] or 0)
        m.plog_numP = I(plog["num_P"])
        m.plog_params = D(plog["post_process"]["params"])
        m.n_cheb = int(cheb["num"])
        pp = np.asarray(cheb["post_process"]["params"])
        m.cheb_maxT = int(pp.shape[1]) if m.n_cheb else 0
        m.cheb_maxP = int(pp.shape[2]) if m.n_cheb else 0
        m.cheb_nT = I(cheb["num_T"])
        m.cheb_nP = I(cheb["num_P"])
        m.cheb_params = D(pp)
        m.cheb_Plim = D(cheb["post_process"]["Plim"])
        m.cheb_Tlim = D(cheb["post_process"]["Tlim"])
        m.thd_type = I(v["thd"]["type"])
        m.thd_off = I(_offsets(v["thd"]["spec_num"]))
        m.thd_spec = I(v["thd"]["spec"])
        m.thd_eff = D(v["thd"]["eff"])
        m.fall_ftype = I(fall["ftype"] if nfall else [])
        m.fall_blend = I(fall["blend"])
        m.fall_type = I(fall["type"])
        m.fall_A = D(fall["A"])
        m.fall_b = D(fall["b"])
        m.fall_Ta = D(fall["Ta"])
        m.fall_troe = I(fall_troe)
        m.fall_sri = I(fall_sri)
        for k in ("a", "T1", "T2", "T3"):
            setattr(m, "troe_" + k, D(fall["troe"][k]))
        for k in ("a", "b", "c", "d", "e"):
            setattr(m, "sri_" + k, D(fall["sri"][k]))
        m.a_lo = D(v["thermo"]["a_lo"])
        m.a_hi = D(v["thermo"]["a_hi"])
        m.T_mid = D(v["thermo"]["T_mid"])
        m.mw_post = D(v["mw_post"])
        m.jac_approx = int(getattr(mech, "jac_type", "exact") == "approximate")
        self._m = m
        self.nn = Ns + 1

    def _call(self, fn, param, phi, out, conp, nthreads):
        param = np.ascontiguousarray(param, dtype=np.float64)
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        rc = fn(ctypes.byref(self._m), phi.shape[0], int(bool(conp)), param.ctypes.data_as(_D),
                phi.ctypes.data_as(_D), out.ctypes.data_as(_D), int(nthreads))
        if rc != 0:
            raise RuntimeError("oracle returned %d" % rc)
        return out

    def op_counts(self, param, phi, kind="jacobian", conp=True):
        """FP64 operations of the reference's formulation per state, averaged
        over the given states (C order): dict of OP_NAMES -> count and
        'flops' = add + mul + div + 2 fma (flop_count.cpp)."""
        lib = getattr(self, "_count_lib", None)
        if lib is None:
            lib = self._count_lib = ctypes.CDLL(build_counter())
            lib.orc_count_ops.restype = ctypes.c_int
            lib.orc_count_ops.argtypes = [ctypes.POINTER(_OrcMech), ctypes.c_int, ctypes.c_long,
                                          ctypes.c_int, _D, _D, ctypes.POINTER(ctypes.c_longlong)]
        param = np.ascontiguousarray(param, dtype=np.float64)
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        n = phi.shape[0]
        c = (ctypes.c_longlong * len(OP_NAMES))()
        rc = lib.orc_count_ops(ctypes.byref(self._m), {"rates": 0, "jacobian": 1}[kind], n,
                               int(bool(conp)), param.ctypes.data_as(_D), phi.ctypes.data_as(_D), c)
        if rc != 0:
            raise RuntimeError("orc_count_ops returned %d" % rc)
        out = {k: c[i] / n for i, k in enumerate(OP_NAMES)}
        out["flops"] = out["add"] + out["mul"] + out["div"] + 2 * out["fma"]
        return out

    def rates_detail(self, param, phi, conp=True):
        """Per state intermediates of the species rates (orc_rates_detail):
        dict of kf, kr (n, nr), Pr, Fi (n, n_fall), wdot, conc (n, ns), dphi
        (n, NN)."""
        fn = self._lib.orc_rates_detail
        fn.restype = ctypes.c_int
        fn.argtypes = [ctypes.POINTER(_OrcMech), ctypes.c_int, ctypes.c_double, _D] + [_D] * 7
        param = np.ascontiguousarray(param, dtype=np.float64)
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        n, nr, ns = phi.shape[0], self.mech.val["Nr"], self.nn - 1
        nf = max(int(self.mech.val["fall"]["num"]), 1)
        out = {"kf": np.empty((n, nr)), "kr": np.empty((n, nr)), "Pr": np.empty((n, nf)),
               "Fi": np.empty((n, nf)), "wdot": np.empty((n, ns)), "dphi": np.empty((n, ns + 1)),
               "conc": np.empty((n, ns))}
        for s in range(n):
            row = {k: np.empty(v.shape[1]) for k, v in out.items()}
            rc = fn(ctypes.byref(self._m), int(bool(conp)), float(param[s]), phi[s].ctypes.data_as(_D),
                    *[row[k].ctypes.data_as(_D) for k in ("kf", "kr", "Pr", "Fi", "wdot", "dphi",
                                                          "conc")])
            if rc != 0:
                raise RuntimeError("oracle returned %d" % rc)
            for k in out:
                out[k][s] = row[k]
        return out

    def species_rates(self, param, phi, conp=True, nthreads=0):
        """phi (n, NN) C order -> dphi (n, NN)."""
        out = np.empty_like(np.asarray(phi, dtype=np.float64))
        return self._call(self._lib.orc_species_rates, param, phi, out, conp, nthreads)

    def rates_scale(self, param, phi, conp=True, nthreads=0):
        """Per-entry cancellation scale of dphi (n, NN); see orc_rates_scale."""
        out = np.empty_like(np.asarray(phi, dtype=np.float64))
        return self._call(self._lib.orc_rates_scale, param, phi, out, conp, nthreads)

    def jacobian(self, param, phi, conp=True, nthreads=0):
        """phi (n, NN) C order -> dense jac (n, NN, NN), jac[i, row, col]."""
        n = np.asarray(phi).shape[0]
        out = np.empty((n, self.nn, self.nn))
        return self._call(self._lib.orc_jacobian, param, phi, out, conp, nthreads)

    def chem_utils(self, phi, conp=True):
        """phi (n, NN) C order -> (cp or cv, h or u, b), each (n, Ns)."""
        phi = np.ascontiguousarray(phi, dtype=np.float64)
        n, ns = phi.shape[0], self.nn - 1
        out = [np.empty((n, ns)) for _ in range(3)]
        rc = self._lib.orc_chem_utils(ctypes.byref(self._m), n, int(bool(conp)), phi.ctypes.data_as(_D),
                                      *[o.ctypes.data_as(_D) for o in out])
        if rc != 0:
            raise RuntimeError("oracle returned %d" % rc)
        return tuple(out)


def _lu_lib():
    lib = ctypes.CDLL(build())
    lib.orc_lu_factor.restype = ctypes.c_int
    lib.orc_lu_factor.argtypes = [ctypes.c_int, ctypes.c_long, ctypes.c_double, _D, ctypes.c_double,
                                  _D, _D, _I, _I]
    lib.orc_lu_solve.restype = ctypes.c_int
    lib.orc_lu_solve.argtypes = [ctypes.c_int, ctypes.c_long, _D, _I, _D]
    lib.orc_lu_sparse_factor.restype = ctypes.c_int
    lib.orc_lu_sparse_factor.argtypes = [ctypes.c_int, ctypes.c_long, ctypes.c_double, _D,
                                         ctypes.c_double, _D, _I, _I, _I, _I, _I, _D, _I]
    lib.orc_lu_sparse_solve.restype = ctypes.c_int
    lib.orc_lu_sparse_solve.argtypes = [ctypes.c_int, ctypes.c_long, _D, _I, _I, _I, _I, _I, _D]
    lib.orc_ros2_combine.restype = ctypes.c_int
    lib.orc_ros2_combine.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_long, _D, ctypes.c_double,
                                     _D, _D, _D, _D, _D]
    return lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(_D)


def lu_factor(jac, s, h):
    """M_i = I - s h_i J_i for jac (n, nn, nn) C order, h scalar or (n,):
    LU with partial pivoting (orc_lu_factor) -> (lu (n, nn, nn), piv (n, nn)
    1-based, info (n,))."""
    jac = np.ascontiguousarray(jac, dtype=np.float64)
    n, nn = jac.shape[0], jac.shape[1]
    lu = np.empty_like(jac)
    piv = np.empty((n, nn), dtype=np.int32)
    info = np.empty(n, dtype=np.int32)
    harr = None if np.ndim(h) == 0 else np.ascontiguousarray(h, dtype=np.float64)
    rc = _lu_lib().orc_lu_factor(nn, n, float(s), _dp(harr), float(h) if harr is None else 0.0,
                                 _dp(jac), _dp(lu), piv.ctypes.data_as(_I), info.ctypes.data_as(_I))
    if rc != 0:
        raise RuntimeError("oracle returned %d" % rc)
    return lu, piv, info


def lu_solve(lu, piv, b):
    """b (n, nn) -> M^-1 b from lu_factor's factors (orc_lu_solve)."""
    lu = np.ascontiguousarray(lu, dtype=np.float64)
    piv = np.ascontiguousarray(piv, dtype=np.int32)
    x = np.array(b, dtype=np.float64, order="C", copy=True)
    rc = _lu_lib().orc_lu_solve(lu.shape[1], lu.shape[0], _dp(lu), piv.ctypes.data_as(_I), _dp(x))
    if rc != 0:
        raise RuntimeError("oracle returned %d" % rc)
    return x


def ros2_combine(op, h, x, k, z=None):
    """ROS2 stage arithmetic (orc_ros2_combine), C order (n, nn) arrays."""
    x = np.ascontiguousarray(x, dtype=np.float64)
    k = np.ascontiguousarray(k, dtype=np.float64)
    z = None if z is None else np.ascontiguousarray(z, dtype=np.float64)
    n, nn = x.shape
    out = np.empty_like(x)
    err = np.empty_like(x) if op == 2 else None
    harr = None if np.ndim(h) == 0 else np.ascontiguousarray(h, dtype=np.float64)
    _lu_lib().orc_ros2_combine(op, nn, n, _dp(harr), float(h) if harr is None else 0.0, _dp(x),
                               _dp(k), _dp(z), _dp(out), _dp(err))
    return (out, err) if op == 2 else out


def lu_plan(row_ptr, col_ind):
    """Static-pivot plan of M = I - s h J for a CRS pattern (plus the
    diagonal): the Markowitz order (at each step the remaining diagonal entry
    with the least (row count - 1) x (column count - 1) over the remaining
    submatrix, lowest index on ties; the pattern fills in as each step
    eliminates), then the symbolic factorisation of the permuted pattern.
    Returns a dict of int32 arrays: perm, roff/ridx (rows below each pivot),
    coff/cidx (columns right of it), loff/lidx and uoff/uidx (the filled L and
    U rows), plus nnz_lu and fma (FMAs per state)."""
    rp = np.asarray(row_ptr)
    ci = np.asarray(col_ind)
    nn = rp.size - 1
    A = np.eye(nn, dtype=bool)
    for r in range(nn):
        A[r, ci[rp[r]:rp[r + 1]]] = True
    done = np.zeros(nn, dtype=bool)
    perm = []
    W = A.copy()
    for _ in range(nn):
        rem = ~done
        best, bscore = -1, None
        for v in np.nonzero(rem)[0]:
            rc = int(W[v, rem].sum()) - 1
            cc = int(W[rem, v].sum()) - 1
            if bscore is None or rc * cc < bscore:
                best, bscore = v, rc * cc
        rows = [r for r in np.nonzero(rem & W[:, best])[0] if r != best]
        cols = [c for c in np.nonzero(rem & W[best, :])[0] if c != best]
        for r in rows:
            W[r, cols] = True
        done[best] = True
        perm.append(int(best))
    perm = np.array(perm, dtype=np.int32)
    B = A[np.ix_(perm, perm)].copy()
    roff, coff, ridx, cidx, fma = [0], [0], [], [], 0
    for k in range(nn):
        R = [r for r in range(k + 1, nn) if B[r, k]]
        C = [c for c in range(k + 1, nn) if B[k, c]]
        for r in R:
            B[r, C] = True
        fma += len(R) * len(C)
        ridx += R
        cidx += C
        roff.append(len(ridx))
        coff.append(len(cidx))
    loff, uoff, lidx, uidx = [0], [0], [], []
    for r in range(nn):
        cols = np.nonzero(B[r])[0]
        lidx += [int(c) for c in cols if c < r]
        uidx += [int(c) for c in cols if c > r]
        loff.append(len(lidx))
        uoff.append(len(uidx))
    a32 = lambda x: np.ascontiguousarray(np.array(x if len(x) else [0], dtype=np.int32))
    return {"perm": perm, "roff": a32(roff), "ridx": a32(ridx), "coff": a32(coff),
            "cidx": a32(cidx), "loff": a32(loff), "lidx": a32(lidx), "uoff": a32(uoff),
            "uidx": a32(uidx), "nnz_lu": int(B.sum()), "fma": fma}


def lu_factor_sparse(jac, s, h, plan):
    """Static-pivot factorisation (orc_lu_sparse_factor) of M_i = I - s h_i J_i,
    jac (n, nn, nn) C order -> (lu of the permuted matrix, info)."""
    jac = np.ascontiguousarray(jac, dtype=np.float64)
    n, nn = jac.shape[0], jac.shape[1]
    lu = np.empty_like(jac)
    info = np.empty(n, dtype=np.int32)
    harr = None if np.ndim(h) == 0 else np.ascontiguousarray(h, dtype=np.float64)
    ip = lambda k: plan[k].ctypes.data_as(_I)
    rc = _lu_lib().orc_lu_sparse_factor(nn, n, float(s), _dp(harr), float(h) if harr is None else 0.0,
                                        _dp(jac), ip("perm"), ip("roff"), ip("ridx"), ip("coff"),
                                        ip("cidx"), _dp(lu), info.ctypes.data_as(_I))
    if rc != 0:
        raise RuntimeError("oracle returned %d" % rc)
    return lu, info


def lu_solve_sparse(lu, b, plan):
    """b (n, nn) -> M^-1 b from lu_factor_sparse's factors (orc_lu_sparse_solve)."""
    lu = np.ascontiguousarray(lu, dtype=np.float64)
    x = np.array(b, dtype=np.float64, order="C", copy=True)
    ip = lambda k: plan[k].ctypes.data_as(_I)
    rc = _lu_lib().orc_lu_sparse_solve(lu.shape[1], lu.shape[0], _dp(lu), ip("perm"), ip("loff"),
                                       ip("lidx"), ip("uoff"), ip("uidx"), _dp(x))
    if rc != 0:
        raise RuntimeError("oracle returned %d" % rc)
    return x


ROS2_GAMMA = 1.7071067811865475  # 1 + 1/sqrt(2)


def ros2_step(oracle, param, phi, h, conp=True, plan=None):
    """One ROS2 step (Verwer, Spee, Blom and Hundsdorfer 1999) with the
    oracle's rates and Jacobian: returns (phi_new, err, info).  With a plan
    (lu_plan) the Newton matrix is factored by the static-pivot sparse LU,
    else with partial pivoting."""
    k1 = oracle.species_rates(param, phi, conp=conp)
    J = oracle.jacobian(param, phi, conp=conp)
    if plan is None:
        lu, piv, info = lu_factor(J, ROS2_GAMMA, h)
        solve = lambda b: lu_solve(lu, piv, b)
    else:
        lu, info = lu_factor_sparse(J, ROS2_GAMMA, h, plan)
        solve = lambda b: lu_solve_sparse(lu, b, plan)
    k1 = solve(k1)
    y1 = ros2_combine(0, h, phi, k1)
    k2 = solve(ros2_combine(1, h, oracle.species_rates(param, y1, conp=conp), k1))
    out, err = ros2_combine(2, h, phi, k1, k2)
    return out, err, info


class RefKernels(object):
    """The reference's shipped generated kernels, shim-compiled into oracle/_ref.

    Available only where ``oracle/build_ref.py`` could compile them (it needs
    the reference tree).  F order in and out, conp, hybrid rate spec.
    """

    def __init__(self, mech_name):
        so = os.path.join(HERE, "_ref", "libref_%s.so" % mech_name)
        if not os.path.exists(so):
            raise FileNotFoundError(so)
        self._lib = ctypes.CDLL(so)
        ns, nn, js = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self._lib.ref_info(ctypes.byref(ns), ctypes.byref(nn), ctypes.byref(js))
        self.ns, self.nn, self.jac_size = ns.value, nn.value, js.value
        for fn in (self._lib.ref_species_rates, self._lib.ref_jacobian):
            fn.restype = ctypes.c_int
            fn.argtypes = [ctypes.c_long, _D, _D, _D, ctypes.c_int]

    @staticmethod
    def available(mech_name):
        return os.path.exists(os.path.join(HERE, "_ref", "libref_%s.so" % mech_name))

    def species_rates_F(self, P, phi_F, nthreads=0):
        n = P.shape[0]
        out = np.zeros((self.nn, n))
        self._lib.ref_species_rates(n, np.ascontiguousarray(P).ctypes.data_as(_D),
                                    np.ascontiguousarray(phi_F).ctypes.data_as(_D),
                                    out.ctypes.data_as(_D), int(nthreads))
        return out

    def jacobian_F(self, P, phi_F, nthreads=0):
        n = P.shape[0]
        out = np.zeros((self.jac_size, n))
        self._lib.ref_jacobian(n, np.ascontiguousarray(P).ctypes.data_as(_D),
                               np.ascontiguousarray(phi_F).ctypes.data_as(_D),
                               out.ctypes.data_as(_D), int(nthreads))
        return out

    def chem_utils_F(self, phi_F, nthreads=0):
        """The shipped chem_utils kernel: (cp, h, b), each (Ns, n) F order."""
        n = phi_F.shape[1]
        out = [np.zeros((self.ns, n)) for _ in range(3)]
        fn = self._lib.ref_chem_utils
        fn.restype = ctypes.c_int
        fn.argtypes = [ctypes.c_long, _D, _D, _D, _D, ctypes.c_int]
        fn(n, np.ascontiguousarray(phi_F).ctypes.data_as(_D), *[o.ctypes.data_as(_D) for o in out],
           int(nthreads))
        return tuple(out)

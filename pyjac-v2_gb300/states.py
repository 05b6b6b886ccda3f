"""Seeded synthetic thermochemical states in pyJac's state layout.

Draws (per state): T ~ U(T_lo, T_hi) K; P = 1 atm * exp(U(ln p_lo, ln p_hi));
mole fractions X ~ Dirichlet(alpha * 1_Ns) over all species including the
bath gas, optionally floored (X <- max(X, floor), renormalised); V = 1 m^3.
Moles n_k = X_k P V / (R_u T).  The state vector follows pyJac
(pyjac/core/array_creator.py:1967-1975): phi = (T, V, n_0 .. n_{Ns-2}) with
param = P at constant pressure, phi = (T, P, n_0 .. n_{Ns-2}) with param = V at
constant volume.
"""
import numpy as np

from .mech.elements import RU, PA


def draw_states(n_species, n, seed=0, T_range=(800.0, 2200.0), p_atm_range=(1.0, 25.0),
                alpha=0.5, x_floor=None, conp=True, order="C", V=1.0):
    """Return (param, phi) as float64 arrays; phi is (n, Ns+1) for order 'C',
    (Ns+1, n) storage (i.e. phi[j, i]) for order 'F'."""
    rng = np.random.default_rng(seed)
    T = rng.uniform(T_range[0], T_range[1], size=n)
    P = PA * np.exp(rng.uniform(np.log(p_atm_range[0]), np.log(p_atm_range[1]), size=n))
    X = rng.dirichlet(alpha * np.ones(n_species), size=n)
    if x_floor is not None:
        X = np.maximum(X, x_floor)
        X /= X.sum(axis=1, keepdims=True)
    Vv = np.full(n, V)
    moles = X * (P * Vv / (RU * T))[:, None]
    phi = np.empty((n, n_species + 1))
    phi[:, 0] = T
    phi[:, 1] = Vv if conp else P
    phi[:, 2:] = moles[:, :-1]
    param = P.copy() if conp else Vv.copy()
    if order == "F":
        phi = np.ascontiguousarray(phi.T)
    return param, phi

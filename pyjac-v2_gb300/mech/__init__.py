"""Mechanism front end: Chemkin reader, pyJac tables, Jacobian sparsity.

``load_mechanism(mech, therm=None, last_spec=None)`` is the entry point: it
parses the mechanism (``chemkin.read_mech``), moves the bath gas last
(``tables.reorder``) and builds the reference-compatible tables and the
Jacobian pattern (``tables.determine_jac_inds``).
"""
import hashlib
import os

import numpy as np

from . import chemkin, tables
from .chemkin import ChemkinError


class Mechanism(object):
    """A parsed mechanism with pyJac-ordered species and its tables.

    Attributes
    ----------
    species : list of chemkin.Species (bath gas last)
    reactions : list of chemkin.Reaction (species as indices)
    val : dict, the reference's assign_rates/determine_jac_inds tables
    """

    def __init__(self, elems, species, reactions, rate_spec="hybrid", jac_type="exact",
                 source=""):
        self.elements = elems
        self.species = species
        self.reactions = reactions
        self.rate_spec = rate_spec
        self.jac_type = jac_type
        self.source = source
        self.val = tables.determine_jac_inds(reactions, species, rate_spec, jac_type)
        for r in reactions:
            for nu in list(r.reac_nu) + list(r.prod_nu):
                if not float(nu).is_integer():
                    raise ChemkinError("non-integer stoichiometric coefficients are not supported "
                                       "by the GPU kernels (reaction %s)" % r.rxn_str)

    @property
    def n_species(self):
        return len(self.species)

    @property
    def n_reactions(self):
        return len(self.reactions)

    @property
    def nn(self):
        """State length: T, extra variable and Ns - 1 species."""
        return len(self.species) + 1

    def species_names(self):
        return [s.name for s in self.species]

    def reaction_strings(self):
        return [r.rxn_str for r in self.reactions]

    @property
    def mw(self):
        return np.asarray(self.val["mws"])

    def jac_nnz(self):
        return int(len(self.val["jac_inds"]["flat_C"]))

    def pattern(self, order="C"):
        """Return (ptr, ind) — CRS (row_ptr, col_ind) for C order, CCS for F."""
        ji = self.val["jac_inds"]
        if order == "C":
            return ji["crs"]["row_ptr"], ji["crs"]["col_ind"]
        return ji["ccs"]["col_ptr"], ji["ccs"]["row_ind"]

    def digest(self):
        """Stable hash of the tables, used to tag checkpoints."""
        h = hashlib.sha256()
        h.update(("|".join(self.species_names()) + "#" + "|".join(self.reaction_strings())).encode())

        def feed(v):
            if isinstance(v, dict):
                for k in sorted(v):
                    feed(v[k])
            elif isinstance(v, np.ndarray) and v.dtype != object:
                h.update(np.ascontiguousarray(v).tobytes())
        feed(self.val)
        return h.hexdigest()[:16]


def load_mechanism(mech, therm=None, last_spec=None, rate_spec="hybrid", jac_type="exact"):
    """Parse a Chemkin mechanism (and optional separate thermo file)."""
    elems, specs, reacs = chemkin.read_mech(mech, therm)
    specs, reacs = tables.reorder(specs, reacs, last_spec)
    return Mechanism(elems, specs, reacs, rate_spec, jac_type, source=os.path.basename(mech))


__all__ = ["Mechanism", "load_mechanism", "ChemkinError", "chemkin", "tables"]

"""The seeded synthetic mechanism generator (the 500-species benchmark
mechanism and the smaller ones the implicit-step tests use)."""
import hashlib
import os
import tempfile

import pytest

from conftest import pkg


@pytest.mark.parametrize("n_species,n_reactions", [(40, 101), (60, 180), (119, 357), (168, 504)])
def test_requested_reaction_count(n_species, n_reactions):
    """Every requested size yields exactly that many reactions; the special
    kinds are rounded one by one and the elementary reactions fill the rest
    (168 species, 504 reactions once came out one short)."""
    path = os.path.join(tempfile.mkdtemp(), "syn.inp")
    pkg("mech.synthetic").write(path, n_species=n_species, n_reactions=n_reactions, seed=5)
    mech = pkg().load_mechanism(path)
    assert mech.n_species == n_species  # the N2 bath gas included
    assert mech.n_reactions == n_reactions


def test_default_mechanism_text_is_stable():
    """The 500-species benchmark mechanism (seed 0) is a fixed text: its
    digest pins the workload that the benchmark numbers refer to."""
    text = pkg("mech.synthetic").generate()
    assert hashlib.md5(text.encode()).hexdigest() == "d3f920cf2133fa9c7ece8e8c88ce6ee9"

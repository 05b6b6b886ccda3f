"""Binary initial-condition files (the reference's read_initial_conditions,
pyjac/kernel_utils/common/read_initial_conditions.cpp.in:30-116) through the
C entry points; host code, no GPU."""
import os

import numpy as np
import pytest

from conftest import pkg

NN = 10


def _states(n, seed=0):
    rng = np.random.default_rng(seed)
    return rng.uniform(1e5, 2e6, n), rng.uniform(0.1, 3000.0, (n, NN))


@pytest.mark.parametrize("order", ["C", "F"])
def test_reads_the_documented_record_layout(tmp_path, order):
    """Records written with numpy in the reference's layout read back into
    param and phi of either order."""
    n = 5000  # more than one 4,096-record block
    P, phi = _states(n)
    rec = np.concatenate([phi[:, :1], P[:, None], phi[:, 1:]], axis=1)
    path = tmp_path / "ics.bin"
    rec.tofile(path)
    got_P, got_phi = pkg("ics").read_initial_conditions(path, n, NN, order)
    assert np.array_equal(got_P, P)
    assert np.array_equal(got_phi if order == "C" else got_phi.T, phi)


@pytest.mark.parametrize("order", ["C", "F"])
def test_write_then_read_round_trip(tmp_path, order):
    ics = pkg("ics")
    P, phi = _states(777, 1)
    x = phi if order == "C" else np.ascontiguousarray(phi.T)
    path = tmp_path / "rt.bin"
    ics.write_initial_conditions(path, P, x, order)
    assert os.path.getsize(path) == 777 * (NN + 1) * 8
    got_P, got_phi = ics.read_initial_conditions(path, 777, NN, order)
    assert np.array_equal(got_P, P) and np.array_equal(got_phi, x)


def test_short_or_missing_file_is_an_error(tmp_path):
    ics = pkg("ics")
    P, phi = _states(10, 2)
    path = tmp_path / "short.bin"
    ics.write_initial_conditions(path, P, phi)
    with pytest.raises(pkg("_lib").PjgError, match="incorrectly formatted"):
        ics.read_initial_conditions(path, 11, NN)
    with pytest.raises(pkg("_lib").PjgError, match="could not open"):
        ics.read_initial_conditions(tmp_path / "missing.bin", 1, NN)
    got_P, got_phi = ics.read_initial_conditions(path, 0, NN)
    assert got_P.size == 0 and got_phi.size == 0

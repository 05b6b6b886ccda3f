"""The benchmark / validation driver with the reference executable's command
line (pyjac-v2_gb300/main.py; kernel.cpp.in:645-750): CSV timing line,
validation output files, and failure on a missing or short data file."""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import DATA, ROOT, load_mech, oracle_mod, pkg

MAIN = os.path.join(ROOT, "pyjac-v2_gb300", "main.py")
GRI = ["--mech", os.path.join(DATA, "grimech30.inp"), "--thermo", os.path.join(DATA, "thermo30.dat")]


def _run(args, cwd):
    return subprocess.run([sys.executable, MAIN] + args, cwd=cwd, capture_output=True, text=True,
                          timeout=600)


def test_missing_data_file_fails(tmp_path):
    r = _run(["16", "1"] + GRI + ["--data", str(tmp_path / "none.bin")], str(tmp_path))
    assert r.returncode != 0
    assert "none.bin" in r.stderr


def test_short_data_file_fails(tmp_path):
    mech = load_mech("gri30")
    P, phi = pkg("states").draw_states(mech.n_species, 8, seed=1, x_floor=1e-12)
    pkg("ics").write_initial_conditions(str(tmp_path / "data.bin"), P, phi)
    r = _run(["16", "1"] + GRI, str(tmp_path))
    assert r.returncode != 0


@pytest.mark.gpu
@pytest.mark.parametrize("kernel,order", [("jacobian", "F"), ("jacobian", "C"), ("species_rates", "C")])
def test_csv_line_and_validation_output(tmp_path, kernel, order):
    mech = load_mech("gri30")
    n = 300
    P, phi = pkg("states").draw_states(mech.n_species, n, seed=14, x_floor=1e-12)
    pkg("ics").write_initial_conditions(str(tmp_path / "data.bin"), P, phi)
    r = _run([str(n), "4"] + GRI + ["--kernel", kernel, "--order", order, "--validate"],
             str(tmp_path))
    assert r.returncode == 0, r.stderr
    fields = r.stdout.strip().splitlines()[-1].split(",")
    assert len(fields) == 4 and int(fields[0]) == n
    assert all(float(f) > 0 for f in fields[1:])
    o = oracle_mod().Oracle(mech)
    NN = mech.nn
    if kernel == "jacobian":
        out = np.fromfile(str(tmp_path / "jac.bin"))
        J = out.reshape(n, NN, NN) if order == "C" else out.reshape(NN, NN, n).transpose(2, 1, 0)
        from conftest import row_rel_err
        assert row_rel_err(J, o.jacobian(P, phi)) < 1e-8
    else:
        d = np.fromfile(str(tmp_path / "dphi.bin")).reshape(n, NN)
        ref = o.species_rates(P, phi)
        den = np.abs(ref) + o.rates_scale(P, phi)
        diff = np.abs(d - ref)
        assert (diff[den == 0] == 0).all()
        assert (diff[den > 0] / den[den > 0]).max() < 1e-10


@pytest.mark.gpu
def test_compile_zero_prints_minus_one(tmp_path):
    mech = load_mech("gri30")
    P, phi = pkg("states").draw_states(mech.n_species, 64, seed=2, x_floor=1e-12)
    pkg("ics").write_initial_conditions(str(tmp_path / "data.bin"), P, phi)
    r = _run(["64", "1", "0"] + GRI, str(tmp_path))
    assert r.returncode == 0, r.stderr
    fields = r.stdout.strip().splitlines()[-1].split(",")
    assert float(fields[1]) == -1.0

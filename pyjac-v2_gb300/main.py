"""Benchmark / validation driver with the command line of the reference's
generated executable (pyjac/kernel_utils/common/kernel.cpp.in:645-750).

    python pyjac-v2_gb300/main.py problem_size work_size [compile] --mech M.inp ...

Reads ``problem_size`` initial conditions from the binary file (default
``data.bin``: records [T, param, phi_1, n_0 .. n_{Ns-2}], C order on disk),
creates the kernel object, evaluates, and prints one line
``problem_size,compile_ms,setup_ms,run_ms`` in the reference's format
(``%zu,%.15le,%.15le,%.15le``, milliseconds, -1 for compile when it is 0) —
the line the reference's performance tester parses
(pyjac/performance_tester/performance_tester.py:130-135).  With
``--validate`` the output is also written as raw doubles in the kernel's data
order to ``jac.bin`` or ``dphi.bin`` (the reference's write_data,
pyjac/kernel_utils/common/write_data.hpp).

"compile" times building the device copy of the mechanism (table packing and
upload: what the reference's OpenCL build of the generated source stands for);
with compile 0 that work is part of setup.  ``work_size`` is accepted and
passed on, as by the reference (the kernel object sizes its own chunks).
"""
import argparse
import importlib
import os
import sys
import time

import numpy as np

PKG = "pyjac-v2_gb300"


def _pkg(sub=None):
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if root not in sys.path:
        sys.path.insert(0, root)
    return importlib.import_module(PKG + ("." + sub if sub else ""))


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("problem_size", type=int)
    ap.add_argument("work_size", type=int)
    ap.add_argument("compile", type=int, nargs="?", default=1)
    ap.add_argument("--mech", required=True, help="Chemkin mechanism file")
    ap.add_argument("--thermo", default=None, help="separate thermo file")
    ap.add_argument("--kernel", default="jacobian", choices=["jacobian", "species_rates"])
    ap.add_argument("--order", default="C", choices=["C", "F"])
    ap.add_argument("--jac-format", default="full", choices=["full", "sparse"])
    ap.add_argument("--conv", action="store_true", help="constant volume (param = V)")
    ap.add_argument("--data", default="data.bin", help="binary initial-condition file")
    ap.add_argument("--validate", action="store_true",
                    help="write the output to jac.bin / dphi.bin in --out-dir")
    ap.add_argument("--out-dir", default=".")
    args = ap.parse_args(argv)
    if args.problem_size < 0 or args.work_size < 0:
        ap.error("sizes must be non-negative")

    mech = _pkg().load_mechanism(args.mech, args.thermo)
    ics = _pkg("ics")
    api = _pkg("api")
    n, nn = args.problem_size, mech.nn
    param, phi = ics.read_initial_conditions(args.data, n, nn, order=args.order)

    mod = api.pywrap(mech, order=args.order, conp=not args.conv, jac_format=args.jac_format)
    cls = mod.PyJacobianKernel if args.kernel == "jacobian" else mod.PySpecies_RatesKernel
    compile_ms = -1.0
    if args.compile:
        t0 = time.perf_counter()
        mod.PyJacobianKernel._dev_mech()
        compile_ms = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    kern = cls(n, args.work_size)
    setup_ms = (time.perf_counter() - t0) * 1e3
    if args.kernel == "jacobian":
        per = nn * nn if args.jac_format == "full" else kern._dm.nnz
    else:
        per = nn
    out = np.empty(n * per)
    t0 = time.perf_counter()
    kern(np.ascontiguousarray(param), phi, out)
    run_ms = (time.perf_counter() - t0) * 1e3
    print("%d,%.15e,%.15e,%.15e" % (n, compile_ms, setup_ms, run_ms))
    if args.validate:
        name = "jac.bin" if args.kernel == "jacobian" else "dphi.bin"
        out.tofile(os.path.join(args.out_dir, name))
    kern.close()
    return 0


if __name__ == "__main__":
    try:
        sys.exit(main())
    except RuntimeError as e:  # library errors: message and a failing status, as the reference's cassert
        print(str(e), file=sys.stderr)
        sys.exit(1)

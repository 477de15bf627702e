"""Extracts the reference's own pinned values for this path into reference_values.json.

Reads the reference test sources as text (run once in the build container, where the
reference tree is mounted; pass its path as argv[1]).  Nothing at test time reads
the reference tree: the tests use the committed JSON.

Sources:
  tests/qmoperators/coulomb_operator.cpp:78-84   <phi_i|J|phi_j>, H n<=2, k=5, prec 1e-3
  tests/qmoperators/exchange_operator.cpp:75-78  <phi_i|K|phi_j>, H 1s/2s, k=5, prec 1e-3
  tests/qmfunctions/density.cpp:68-69,79-80      int rho = 7 / 3 / 5 / 2
  tests/unit_tests.cpp:66-84                     MRA fixture
The analytic hydrogenic Slater integrals (Z = 1) are added for the continuum check.
"""
import json
import os
import re
import sys


def ep_values(path):
    vals = {}
    for m in re.finditer(r"E_P\((\d+),\s*(\d+)\)\s*=\s*([0-9.eE+-]+);", open(path).read()):
        vals["%s,%s" % (m.group(1), m.group(2))] = float(m.group(3))
    return vals


def main(ref):
    out = {
        "mra": {"order": 5, "basis": "interpolating", "root_scale": -5, "corner": [-1, -1, -1], "boxes": [2, 2, 2],
                "max_depth": 25, "source": "tests/unit_tests.cpp:66-84"},
        "coulomb": {"prec": 1e-3, "orbitals": [[1, 0, 0], [2, 0, 0], [2, 1, 0], [2, 1, 1], [2, 1, 2]],
                    "occupation": 2.0, "E_P": ep_values(os.path.join(ref, "tests/qmoperators/coulomb_operator.cpp")),
                    "source": "tests/qmoperators/coulomb_operator.cpp:78-84"},
        "exchange": {"prec": 1e-3, "orbitals": [[1, 0, 0], [2, 0, 0]],
                     "E_P": ep_values(os.path.join(ref, "tests/qmoperators/exchange_operator.cpp")),
                     "source": "tests/qmoperators/exchange_operator.cpp:75-78"},
        "density": {"prec": 1e-3, "total": 7.0, "spin": 3.0, "alpha": 5.0, "beta": 2.0,
                    "source": "tests/qmfunctions/density.cpp:68-69,79-80"},
        "analytic": {"J_1s1s": 5.0 / 8.0, "J_1s2s": 17.0 / 81.0, "J_1s2p": 59.0 / 243.0, "J_2s2s": 77.0 / 512.0,
                     "K_1s2s": 16.0 / 729.0,
                     "coulomb_00_closed_shell": 2 * (5.0 / 8.0 + 17.0 / 81.0 + 3 * 59.0 / 243.0),
                     "exchange_00": 5.0 / 8.0 + 16.0 / 729.0, "exchange_11": 16.0 / 729.0 + 77.0 / 512.0},
    }
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "reference_values.json"), "w") as f:
        json.dump(out, f, indent=1, sort_keys=True)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")

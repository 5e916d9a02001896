"""Copies the reference's golden trajectories for the ODE-SECIR path into
tests/golden/ so that the tests can run where the reference is absent.

Sources (read-only reference tree):
  pycode/memilio-simulation/tests/data/ode-secihurd-compare.csv        (test_osecir.py:122-150, default Cash-Karp)
  pycode/memilio-simulation/tests/data/ode-secihurd-ageres-compare.csv (test_osecir_ageres.py:116-145, default Cash-Karp)
  cpp/tests/data/secihurd-compare-cashkarp.csv (test_odesecir_ageres.cpp:110-189, bounded Cash-Karp)
  cpp/tests/data/secihurd-compare.csv          (test_odesecir.cpp:39-112, test_odesecir_ageres.cpp:27-108, RKF45)

Usage: python tests/golden/make_golden.py <reference_root>
(the root of the MEmilio source tree, the directory holding cpp/ and pycode/)
"""
import os
import shutil
import sys

FILES = [
    "pycode/memilio-simulation/tests/data/ode-secihurd-compare.csv",
    "pycode/memilio-simulation/tests/data/ode-secihurd-ageres-compare.csv",
    "cpp/tests/data/secihurd-compare-cashkarp.csv",
    "cpp/tests/data/secihurd-compare.csv",
]


def main():
    if len(sys.argv) != 2:
        sys.exit(__doc__)
    root = sys.argv[1]
    here = os.path.dirname(os.path.abspath(__file__))
    for rel in FILES:
        shutil.copyfile(os.path.join(root, rel), os.path.join(here, os.path.basename(rel)))
        print("copied", rel)


if __name__ == "__main__":
    main()

"""Copies the reference's own CI fixtures into tests/golden/ci/.

The reference pins its forward solver with golden seismograms
(par/ci/seismogram.*.ref.*.mtx) produced by its CI configurations
(par/ci/configuration_ci.*.txt, sources_ci.*.txt, receiver_ci.*.txt) and checked
by src/Tests/IntegrationTest/Test_CompareSeismogram.cpp. The reference tree is
not available where the GPU tests run, so the files are committed here as
fixtures. Run from the repository root:

    python tests/golden/make_fixtures.py /path/to/reference
"""
import os
import shutil
import sys

DST = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ci")

KEEP_PREFIX = ("configuration_ci.", "sources_ci.", "receiver_ci.", "seismogram.")


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_fixtures.py <path of the reference checkout>")
    SRC = os.path.join(sys.argv[1], "par", "ci")
    os.makedirs(DST, exist_ok=True)
    n = 0
    for name in sorted(os.listdir(SRC)):
        if name.startswith(KEEP_PREFIX) or name == "gridConfig.txt":
            shutil.copyfile(os.path.join(SRC, name), os.path.join(DST, name))
            n += 1
    print(f"copied {n} fixture files into {DST}")


if __name__ == "__main__":
    main()

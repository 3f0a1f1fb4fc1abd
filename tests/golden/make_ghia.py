"""Centre-line velocity profiles of the 2D lid-driven cavity at Re 1000 (Ghia, Ghia
and Shin, J. Comput. Phys. 48, 1982), as the reference ships them for its 2D cavity
check (tests/ldcTest/u_profile_ghia.dat, v_profile_ghia.dat): u along the vertical
centre line against the height, w along the horizontal centre line against x.

    python tests/golden/make_ghia.py [path of the reference checkout]

writes tests/golden/ghia_re1000.npz (arrays z, u, x, w)."""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def read(path):
    rows = []
    for line in open(path):
        line = line.strip()
        if not line or line.startswith("#"):
            continue
        _, pos, val = line.split()[:3]
        rows.append((float(pos), float(val)))
    rows.sort()
    return np.array([r[0] for r in rows]), np.array([r[1] for r in rows])


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    d = os.path.join(ref, "tests", "ldcTest")
    z, u = read(os.path.join(d, "u_profile_ghia.dat"))
    x, w = read(os.path.join(d, "v_profile_ghia.dat"))
    out = os.path.join(HERE, "ghia_re1000.npz")
    np.savez(out, z=z, u=u, x=x, w=w)
    print("wrote %s: %d u points, %d w points" % (out, len(z), len(x)))


if __name__ == "__main__":
    main()

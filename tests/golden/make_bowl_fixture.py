"""Packs the reference's only golden data into tests/golden/bowl_euler.npz.

Source (read at generation time only): the reference's notebooks/geometry.dat,
notebooks/topology.dat (mesh written by examples/Main.cpp:126-170 for
examples/bowl.msh with a flat bed) and notebooks/out0.dat / out1.dat (w, hu, hv
per cell before and after one Euler step of HLL + Einfeldt with dt = 1e-3,
examples/Main.cpp:172-195), printed with 6 significant digits.

Usage: python tests/golden/make_bowl_fixture.py <reference root>
"""
import os
import sys

import numpy as np

if len(sys.argv) != 2:
    sys.exit("usage: python tests/golden/make_bowl_fixture.py <reference root>")
root = sys.argv[1]
nb = os.path.join(root, "notebooks")
geo = np.loadtxt(os.path.join(nb, "geometry.dat")).reshape(-1, 3)
lines = open(os.path.join(nb, "topology.dat")).read().split("\n")
E = int(lines[0])
ed = np.array([[int(v) for v in lines[1 + e].split()] for e in range(E)], dtype=np.int32)
C = int(lines[1 + E])
cd = np.array([[int(v) for v in lines[2 + E + c].split()] for c in range(C)], dtype=np.int32)
out0 = np.loadtxt(os.path.join(nb, "out0.dat"))
out1 = np.loadtxt(os.path.join(nb, "out1.dat"))
dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "bowl_euler.npz")
np.savez_compressed(dst, geometry=geo, edges=ed, cells=cd, out0=out0, out1=out1)
print(dst, os.path.getsize(dst))

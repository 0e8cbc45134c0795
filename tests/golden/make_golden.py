"""Generates tests/golden/tiny_dome.npz with the CPU oracle.

The reference (Fortran 90 + MPI + netCDF) cannot be built or run here and ships no golden
vectors, so this fixture pins the oracle against itself across machines and over time: the
Ac / AaAc mesh arrays and the five-colouring of the seeded "tiny" dome mesh, the AaAc
neighbour functions, and one cold-start SSA solve (linear sliding) and SIA solve on it.

Run:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

import oracle as orc  # noqa: E402
from conftest import oracle_aaac, oracle_inputs  # noqa: E402


def main():
    m = oracle_aaac("tiny")
    ssa, sia, g = oracle_inputs(m)
    rc, out, st = orc.solve_ssa(m, ssa, orc.default_params())
    so = orc.solve_sia(m, sia, orc.default_params())
    arrs = {k: np.asarray(getattr(m, k)) for k in ("iAci", "Aci", "edge_index_Ac", "nCAaAc", "CAaAc", "colour",
                                                   "colour_vi", "colour_nV", "Nx_AaAc", "Ny_AaAc", "Nxx_AaAc",
                                                   "Nxy_AaAc", "Nyy_AaAc")}
    arrs.update(U_SSA=out["U_SSA"], V_SSA=out["V_SSA"], Ux_SSA_Ac=out["Ux_SSA_Ac"], Uy_SSA_Ac=out["Uy_SSA_Ac"],
                sweeps=np.array(st["sweeps"], dtype=np.int32), Ux_SIA_Ac=so["Ux_SIA_Ac"])
    np.savez_compressed(os.path.join(HERE, "tiny_dome.npz"), **arrs)
    print("rc", rc, "stats", st)


if __name__ == "__main__":
    main()

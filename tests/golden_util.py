"""Loaders for the committed golden fixtures (tests/golden/*.npz), made by
tests/golden/make_golden.py from the reference's own code."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=True)


def eri_cases():
    """Yields (l[4], pure[4], nprim[4], alpha, coeff, O[12], deriv, values)."""
    g = load("eri.npz")
    offs = list(g["offset"]) + [len(g["values"])]
    for i in range(len(g["l"])):
        n = int(g["nprim"][i].sum())
        yield (g["l"][i], g["pure"][i], g["nprim"][i], g["alpha"][i][:n], g["coeff"][i][:n],
               g["O"][i], int(g["deriv"][i]), g["values"][offs[i]:offs[i + 1]])


def eri3c_cases():
    """Yields (l[4], pure[4], nprim[4], alpha, coeff, O[12], deriv, rank, values)
    of the 3-/2-centre fixtures (unit shells in positions 1, and 3 for rank 2;
    values hold all 12 derivative sets for deriv 1)."""
    g = load("eri3c.npz")
    offs = list(g["offset"]) + [len(g["values"])]
    for i in range(len(g["l"])):
        n = int(g["nprim"][i].sum())
        yield (g["l"][i], g["pure"][i], g["nprim"][i], g["alpha"][i][:n], g["coeff"][i][:n],
               g["O"][i], int(g["deriv"][i]), int(g["rank"][i]),
               g["values"][offs[i]:offs[i + 1]])


def eri_d2_cases():
    """Yields (l[4], pure[4], nprim[4], alpha, coeff, O[12], values[78*n]) of
    the second-derivative fixtures; load("eri_d2.npz")["c1"/"c2"] hold the
    reference's set order."""
    g = load("eri_d2.npz")
    offs = list(g["offset"]) + [len(g["values"])]
    for i in range(len(g["l"])):
        n = int(g["nprim"][i].sum())
        yield (g["l"][i], g["pure"][i], g["nprim"][i], g["alpha"][i][:n], g["coeff"][i][:n],
               g["O"][i], g["values"][offs[i]:offs[i + 1]])

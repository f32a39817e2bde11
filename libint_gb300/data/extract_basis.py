"""Extracts the first-row-element blocks (H..Ne) of a few G94 basis-set
library files shipped with the reference (lib/basis/*.g94) into
libint_gb300/data/basis/, so the package carries the basis data it needs
(cc-pVDZ, cc-pVTZ, their aug- augmentations, 6-31G, STO-3G) without the
reference tree.  The numbers are the EMSL Basis Set Exchange data those
files redistribute; the header comments (citations) are kept.

usage: python libint_gb300/data/extract_basis.py [REFERENCE_ROOT]
"""
import os
import sys

NAMES = ["cc-pvdz", "cc-pvtz", "augmentation-cc-pvdz", "augmentation-cc-pvtz",
         "6-31g", "sto-3g", "cc-pvdz-jkfit"]
KEEP = {"H", "He", "Li", "Be", "B", "C", "N", "O", "F", "Ne"}


def extract(src, dst):
    out, block, elem, header = [], [], None, True
    with open(src) as f:
        lines = f.read().splitlines()
    i = 0
    for line in lines:
        if header:
            if line.strip() == "****":
                header = False
                out.append(line)
                continue
            out.append(line)
            continue
        if elem is None:
            if not line.strip() or line.startswith("!"):
                continue
            elem = line.split()[0]
            block = [line]
            continue
        block.append(line)
        if line.strip() == "****":
            if elem in KEEP:
                out.extend(block)
            elem, block = None, []
    with open(dst, "w") as f:
        f.write("\n".join(out) + "\n")


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("LGX_REFERENCE_ROOT")
    if not ref:
        sys.exit("usage: extract_basis.py LIBINT_TREE  (or set LGX_REFERENCE_ROOT)")
    here = os.path.join(os.path.dirname(os.path.abspath(__file__)), "basis")
    os.makedirs(here, exist_ok=True)
    for n in NAMES:
        extract(os.path.join(ref, "lib", "basis", n + ".g94"), os.path.join(here, n + ".g94"))
        print("wrote", n)


if __name__ == "__main__":
    main()

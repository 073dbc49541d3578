"""Write the H/C/N/O subset of the Basis Set Exchange JSON files used by the
DF Fock-build workloads (cc-pVDZ, cc-pVDZ-jkfit, cc-pVDZ-RI, STO-3G).

The data are Basis Set Exchange records (https://www.basissetexchange.org,
Pritchard et al., J. Chem. Inf. Model. 59, 4814 (2019)); the same files ship
with megalochem under basis/*.json.  Only the element entries and the fields
the basis reader uses ("angular_momentum", "exponents", "coefficients") are
kept, as the original strings.

Usage:  python extract_subset.py <dir holding the full BSE JSON files>
"""
import json
import os
import sys

NAMES = ["cc-pvdz", "cc-pvdz-jkfit", "cc-pvdz-ri", "sto-3g"]
ELEMENTS = ["1", "6", "7", "8"]


def main(src):
    here = os.path.dirname(os.path.abspath(__file__))
    for name in NAMES:
        with open(os.path.join(src, name + ".json")) as f:
            full = json.load(f)
        out = {
            "name": full.get("name", name),
            "source": "Basis Set Exchange (basissetexchange.org); subset H, C, N, O",
            "elements": {},
        }
        for z in ELEMENTS:
            shells = []
            for sh in full["elements"][z]["electron_shells"]:
                shells.append({
                    "angular_momentum": sh["angular_momentum"],
                    "exponents": sh["exponents"],
                    "coefficients": sh["coefficients"],
                })
            out["elements"][z] = {"electron_shells": shells}
        with open(os.path.join(here, name + ".json"), "w") as f:
            json.dump(out, f, indent=1)
        print("wrote", name)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference/basis")

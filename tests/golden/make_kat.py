"""Extract the reference's hot-path known-answer values into kat.json.

Reads the doctest sources of the Faunus source tree given as the one
command-line argument (`python make_kat.py <faunus tree>`) as TEXT, checks that each cited line still holds
the expected statement, and writes the numbers with their file:line
provenance.  The tests read only kat.json.
"""
import json
import re
import sys
from pathlib import Path

if len(sys.argv) != 2:
    raise SystemExit("usage: python make_kat.py <path of a Faunus source tree>")
ROOT = Path(sys.argv[1])
NUM = r"(-?\d+\.\d+(?:[eE]-?\d+)?)"

# (key, file, line, regex with one capture group)
ITEMS = [
    ("ewald_kvectors_pbc", "src/energy.cpp", 90, r"k_vectors\.cols\(\), (\d+)\)"),
    ("ewald_kvectors_ipbc", "src/energy.cpp", 97, r"k_vectors\.cols\(\), (\d+)\)"),
    ("ewald_alpha", "src/energy.cpp", 80, r'"alpha": ' + NUM),
    ("ewald_self_per_lB", "src/energy.cpp", 276, r"Approx\(" + NUM),
    ("ewald_surface_per_lB", "src/energy.cpp", 278, r"Approx\(" + NUM),
    ("ewald_reciprocal_pbc_per_lB", "src/energy.cpp", 279, r"Approx\(" + NUM),
    ("ewald_reciprocal_ipbc_per_lB", "src/energy.cpp", 304, r"reciprocalEnergy\(data\), Approx\(" + NUM),
    ("ewald_energy_after_move", "src/energy.cpp", 698, r"Approx\(" + NUM),
    ("ewald_energy_change", "src/energy.cpp", 685, r"energy_change = " + NUM),
    ("lj_force_x", "src/potentials.cpp", 778, r"Approx\(" + NUM),
    ("coulomb_lB_epsr80", "src/potentials.cpp", 660, r"Approx\(" + NUM),
    ("coulomb_force_norm", "src/potentials.cpp", 661, r"Approx\(" + NUM),
    ("newcoulombgalore_plain_force_z", "src/potentials.cpp", 1625, r"Approx\(" + NUM),
]


def main() -> None:
    out = {}
    for key, rel, line, rx in ITEMS:
        text = (ROOT / rel).read_text().splitlines()
        hit = None
        for ln in (line, line + 1, line - 1, line + 2, line - 2):  # exact line first, then +-2 of drift
            m = re.search(rx, text[ln - 1])
            if m:
                hit = (ln, m.group(1))
                break
        if hit is None:
            raise SystemExit(f"{key}: pattern not found near {rel}:{line}")
        ln, val = hit
        out[key] = {"value": float(val) if "." in val or "e" in val else int(val), "source": f"{rel}:{ln}"}
    dst = Path(__file__).with_name("kat.json")
    dst.write_text(json.dumps(out, indent=2) + "\n")
    print(f"wrote {dst} ({len(out)} values)")


if __name__ == "__main__":
    main()

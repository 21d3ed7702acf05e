"""Extract the reference's example runs into compact fixtures.

Reads, as data, from the Faunus source tree given as the one command-line argument
(`python make_example_fixtures.py <faunus tree>`):

  examples/bulk: bulk.yml (the input, converted with the package's YAML reader),
    bulk.state.json (the state the run saved at its end) and bulk.out.json (its output:
    Bjerrum length and the final energies of the particle-self-energy and nonbonded
    terms) -> bulk_example.json (input + expected values with provenance) and
    bulk_example_state.npz (particle ids, positions, charges);
  examples/minimal: minimal.yml and minimal.out.json (SystemEnergy mean over its run, the
    statistical fixture) -> minimal_example.json;
  examples/langevin: montecarlo_lj.yml, montecarlo_lj.out.json and rdf_mc.dat (the AtomRDF
    g(r) its MC run wrote) -> montecarlo_lj_example.json;
  examples/multipole: multipole.state.ubj (a state file the reference wrote as Universal Binary
    JSON) -> multipole.state.ubj, byte for byte (the UBJSON reader and writer are pinned on it);
  examples/cluster: cluster.yml (nonbonded_splined water; its molecule structure read from
    water.xyz into the input, its cluster move and analyses other than SystemEnergy left out),
    cluster.state.json (the state its run started from) and cluster.out.json (SystemEnergy at
    that start, 2 decimals) -> cluster_example.json.

The tests read only the written files.
"""
import json
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parents[1]))
from faunus_gb300 import yason  # noqa: E402

if len(sys.argv) != 2:
    raise SystemExit("usage: python make_example_fixtures.py <path of a Faunus source tree>")
ROOT = Path(sys.argv[1])


def main() -> None:
    ex = ROOT / "examples" / "bulk"
    inp = yason.loads((ex / "bulk.yml").read_text())
    state = json.loads((ex / "bulk.state.json").read_text())
    out = json.loads((ex / "bulk.out.json").read_text())
    nb = out["energy"][0]["hamiltonian"][1]["nonbonded"]
    coul = next(p["coulomb"] for p in nb["pairpot"] if "coulomb" in p)
    final = next(a["systemenergy"]["final"] for a in out["analysis"] if "systemenergy" in a)
    fixture = {
        "provenance": {"input": "examples/bulk/bulk.yml", "state": "examples/bulk/bulk.state.json",
                       "output": "examples/bulk/bulk.out.json", "git revision": out["git revision"],
                       "compiler": out["compiler"]},
        "input": inp,
        "geometry": state["geometry"],
        "groups": state["groups"],
        "expected": {"bjerrum_length": coul["lB"], "self": final[0], "nonbonded": final[1],
                     "temperature": out["temperature"]},
    }
    (HERE / "bulk_example.json").write_text(json.dumps(fixture, indent=1))
    parts = state["particles"]
    mex = ROOT / "examples" / "minimal"
    mout = json.loads((mex / "minimal.out.json").read_text())
    se = next(a["systemenergy"] for a in mout["analysis"] if "systemenergy" in a)
    mv = mout["moves"][0]["transrot"]
    fpot = mout["energy"][0]["hamiltonian"][1]["nonbonded"]["pairpot"]["functor potential"]["default"]
    mlb = next(t["coulomb"]["lB"] for t in fpot if "coulomb" in t)
    (HERE / "minimal_example.json").write_text(json.dumps({
        "provenance": {"input": "examples/minimal/minimal.yml", "output": "examples/minimal/minimal.out.json",
                       "git revision": mout["git revision"], "compiler": mout["compiler"]},
        "input": yason.loads((mex / "minimal.yml").read_text()),
        "expected": {"bjerrum_length": mlb, "systemenergy_mean": se["mean"], "systemenergy_samples": se["samples"],
                     "systemenergy_nstep": se["nstep"], "moves": mv["moves"], "acceptance": mv["acceptance"],
                     "temperature": mout["temperature"]},
    }, indent=1))
    lex = ROOT / "examples" / "langevin"
    lout = json.loads((lex / "montecarlo_lj.out.json").read_text())
    rdf = next(a["atomrdf"] for a in lout["analysis"] if "atomrdf" in a)
    table = [[float(x) for x in line.split()] for line in (lex / "rdf_mc.dat").read_text().splitlines()
             if line.strip() and not line.startswith("#")]
    lmv = lout["moves"][0]["transrot"]
    (HERE / "montecarlo_lj_example.json").write_text(json.dumps({
        "provenance": {"input": "examples/langevin/montecarlo_lj.yml", "output": "examples/langevin/montecarlo_lj.out.json",
                       "rdf": "examples/langevin/rdf_mc.dat", "git revision": lout["git revision"]},
        "input": yason.loads((lex / "montecarlo_lj.yml").read_text()),
        "expected": {"rdf_samples": rdf["samples"], "dr": rdf["dr"], "nstep": rdf["nstep"], "moves": lmv["moves"],
                     "acceptance": lmv["acceptance"], "rdf": table},
    }))
    cex = ROOT / "examples" / "cluster"
    cinp = yason.loads((cex / "cluster.yml").read_text())
    xyz = (cex / "water.xyz").read_text().split("\n")
    natoms = int(xyz[0].split()[0])
    structure = []
    for line in xyz[2:2 + natoms]:
        name, x, y, z = line.split()[:4]
        structure.append({name: [float(x), float(y), float(z)]})
    for item in cinp["moleculelist"]:
        for name, props in item.items():
            if props.get("structure") == "water.xyz":
                props["structure"] = structure
    cinp["moves"] = [m for m in cinp["moves"] if "moltransrot" in m]
    cinp["analysis"] = [a for a in cinp["analysis"] if "systemenergy" in a]
    cout = json.loads((cex / "cluster.out.json").read_text())
    cstate = json.loads((cex / "cluster.state.json").read_text())
    cse = next(a["systemenergy"] for a in cout["analysis"] if "systemenergy" in a)
    cnb = cout["energy"][0]["hamiltonian"][0]["nonbonded"]
    ccoul = next(p["coulomb"] for p in cnb["pairpot"] if "coulomb" in p)
    (HERE / "cluster_example.json").write_text(json.dumps({
        "provenance": {"input": "examples/cluster/cluster.yml (+ water.xyz; cluster move and other analyses "
                                "left out)", "state": "examples/cluster/cluster.state.json",
                       "output": "examples/cluster/cluster.out.json", "git revision": cout["git revision"],
                       "compiler": cout["compiler"]},
        "input": cinp,
        "state": cstate,
        "expected": {"bjerrum_length": ccoul["lB"], "systemenergy_init": cse["init"],
                     "temperature": cout["temperature"]},
    }, indent=1))
    np.savez_compressed(HERE / "bulk_example_state.npz",
                        id=np.array([p["id"] for p in parts], dtype=np.int32),
                        pos=np.array([p["pos"] for p in parts], dtype=np.float64),
                        q=np.array([p["q"] for p in parts], dtype=np.float64))


def copy_state_ubj() -> None:
    (HERE / "multipole.state.ubj").write_bytes((ROOT / "examples" / "multipole" / "multipole.state.ubj").read_bytes())


if __name__ == "__main__":
    main()
    copy_state_ubj()

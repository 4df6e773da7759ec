"""Regenerate tests/golden/lattice_reference.json from the reference's own lattice code.

The reference's `quantax.sites` package uses numpy only, apart from the PARTICLE_TYPE enum of
its `global_defs` module, which imports JAX (absent here). This script registers an empty
`quantax` package whose search path is the reference's source directory and a `global_defs`
stand-in holding an enum with the same member names and values (0 spin, 1 spinful_fermion,
2 spinless_fermion), then imports `quantax.sites` from the reference checkout unchanged. It
records, for the lattices the tests and the bench use, the site coordinates and the n-th
nearest-neighbour bond lists that `Sites.get_neighbor` returns (quantax/sites/sites.py:224-283),
the bonds from which the Heisenberg and J1-J2 operators are built
(quantax/operator/common_operators.py:23-53).

    python tests/golden/make_lattice_golden.py [path-to-reference-checkout]
"""
import enum
import importlib
import json
import sys
import types
from pathlib import Path

HERE = Path(__file__).resolve().parent

CASES = [("Chain", 8, [1, 2]), ("Chain", 16, [1, 2]), ("Chain", 64, [1]), ("Square", 4, [1, 2, 3]),
         ("Square", 6, [1, 2]), ("Square", 10, [1, 2])]


def load_reference_sites(ref: Path):
    pkg = types.ModuleType("quantax")
    pkg.__path__ = [str(ref / "quantax")]
    defs = types.ModuleType("quantax.global_defs")
    defs.PARTICLE_TYPE = enum.Enum("PARTICLE_TYPE", {"spin": 0, "spinful_fermion": 1, "spinless_fermion": 2})
    sys.modules["quantax"] = pkg
    sys.modules["quantax.global_defs"] = defs
    return importlib.import_module("quantax.sites")


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_lattice_golden.py <path of the quantax checkout>")
    ref = Path(sys.argv[1])
    sites = load_reference_sites(ref)
    out = {}
    for kind, L, shells in CASES:
        sites.Sites._SITES = None
        lat = getattr(sites, kind)(L)
        nb = lat.get_neighbor(shells)
        out[f"{kind}({L})"] = {
            "coord": lat.coord.tolist(),
            "neighbors": {str(n): b.tolist() for n, b in zip(shells, nb)},
        }
    (HERE / "lattice_reference.json").write_text(json.dumps(out, separators=(",", ":")))
    print(f"wrote {len(out)} lattices")


if __name__ == "__main__":
    main()

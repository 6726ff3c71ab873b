"""Generate the committed golden fixtures under tests/golden/.

Run where the reference sources are available, giving their root as the
first argument or in $MO_DMFT_REFERENCE (there is no default); the tests
only read the JSON files written here.

notebook_hmat.json
    The reference's only known-answer test: the 9x9 Hamiltonian matrix that
    mathematica/MO-DMFT-ED.nb prints (:1558-1590) for 2 orbitals + 1 bath
    with e1=e2=0, J=200, U=400, mu=100, eb1=0.5, v13=20, v23=10 (:1498-1505),
    in the notebook's 9-state basis `bs` (:1045-1072).  The notebook's
    occupation vector vc[n1..n6] lists (orb1 up, orb1 dn, orb2 up, orb2 dn,
    bath up, bath dn).
"""
import json
import os
import re

REF = None   # the reference's root: first argument or $MO_DMFT_REFERENCE
HERE = os.path.dirname(os.path.abspath(__file__))


def _cells_after(text, anchor, count):
    i = text.index(anchor)
    return text[i:i + 20000]


def parse_notebook():
    nb = open(os.path.join(REF, "mathematica", "MO-DMFT-ED.nb")).read()
    # --- basis bs ---
    i = nb.index('RowBox[{"bs", "="')
    chunk = nb[i:i + 3000]
    vcs = re.findall(r'RowBox\[\{"vc", "\[", \s*RowBox\[\{([^\]]*)\}\], "\]"\}\]', chunk)
    basis = [[int(t) for t in re.findall(r'"(\d)"', v)] for v in vcs]
    assert len(basis) == 9 and all(len(b) == 6 for b in basis), basis
    # --- numeric Hmat (GridBox after the parameter cell) ---
    j = nb.index('RowBox[{"v23", "=", "10"}]')
    k = nb.index("GridBox[{", j)
    end = nb.index("GridBoxAlignment", k)
    grid = nb[k:end]
    rows = []
    for row in re.findall(r"\{\s*(.*?)\}(?=,\s*\{|\s*\},\s*$|\s*\})", grid[len("GridBox[{"):], re.S):
        toks = re.findall(r'RowBox\[\{"-", "([0-9.`]+)"\}\]|"([0-9.`-]+)"', row)
        vals = []
        for neg, pos in toks:
            s = (("-" + neg) if neg else pos).replace("`", "")
            vals.append(float(s))
        if vals:
            rows.append(vals)
    rows = [r for r in rows if len(r) == 9]
    assert len(rows) == 9, [len(r) for r in rows]
    return basis, rows


def main():
    basis, hmat = parse_notebook()
    out = {
        "source": "mathematica/MO-DMFT-ED.nb:1045-1072 (basis), :1498-1505 (parameters), :1558-1590 (Hmat)",
        "params": {"e1": 0.0, "e2": 0.0, "J": 200.0, "U": 400.0, "mu": 100.0, "eb1": 0.5,
                   "v13": 20.0, "v23": 10.0},
        "model": {"norb": 2, "nbath": 1, "U": 400.0, "J": 200.0,
                  "ek": [-100.0, -100.0, 0.5], "vk": [[20.0], [10.0]]},
        "sector": {"ne_up": 2, "ne_down": 1},
        "vc_order": ["orb1_up", "orb1_dn", "orb2_up", "orb2_dn", "bath_up", "bath_dn"],
        "basis_vc": basis,
        "hmat": hmat,
    }
    with open(os.path.join(HERE, "notebook_hmat.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote notebook_hmat.json")


if __name__ == "__main__":
    import sys
    REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MO_DMFT_REFERENCE")
    if not REF:
        sys.exit("usage: make_golden.py REFERENCE_ROOT  (or set MO_DMFT_REFERENCE)")
    main()

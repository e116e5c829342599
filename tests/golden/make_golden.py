"""Generate the golden fixtures under tests/golden/ from the reference's own tests.

Run where the reference project is checked out, giving its root directory as the
first argument or in MCPHYLO_REFERENCE:

    python tests/golden/make_golden.py <path to MCPhylo.jl>

It reads the reference's test files as text:

* test/likelihood/felsenstein.jl:2-41   -> Newick strings, logL and gradient goldens
* test/likelihood/{primates,simudata}.nex -> the alignments (stored as taxon names +
  one ASCII row per taxon; no other transformation)
* test/likelihood/substitutionmodels.jl  -> U, D, Uinv, mu targets of each model
* test/likelihood/rates.jl               -> discrete-Gamma targets
* test/distributions/phylodist.jl:133-135 -> MultiplePhyloDist = 2 x golden

and writes golden.json (numbers) plus one .json per alignment.  The fixtures are
committed; tests never read the reference at run time.
"""
import json
import os
import re
import sys

REF = None   # the reference's root directory, set by main()
OUT = os.path.dirname(os.path.abspath(__file__))


def read(rel):
    with open(os.path.join(REF, rel)) as f:
        return f.read()


def nums(s):
    return [float(t) for t in re.findall(r"-?\d+\.?\d*(?:e-?\d+)?", s)]


def matrix(s):
    """Julia matrix literal '[a b; c d]' -> list of rows."""
    s = s.strip().strip("[]")
    return [nums(row) for row in s.split(";")]


def alignment(rel):
    lines = read(rel).splitlines()
    i = next(k for k, ln in enumerate(lines) if "matrix" in ln.lower())
    taxa, rows = [], []
    for ln in lines[i + 1:]:
        if ln.strip() == "":
            continue
        if ln.rstrip()[-1] == ";":
            break
        name, raw = ln.split(None, 1)
        taxa.append(name)
        rows.append(raw.strip())
    return {"source": rel, "taxa": taxa, "rows": rows}


def main():
    fel = read("test/likelihood/felsenstein.jl")
    newicks = re.findall(r'ParseNewick\(\s*"(.*?)"', fel, flags=re.S)
    prim_ll = float(re.search(r"logpdf\(pd, df\) ≈ (-?[\d.]+)", fel).group(1))
    sim_ll = float(re.search(r"ll = (-?[\d.]+)", fel).group(1))
    sim_grad = nums(re.search(r"grad = \[(.*?)\]", fel, flags=re.S).group(1))

    sub = read("test/likelihood/substitutionmodels.jl")
    restr = re.search(r"target = \((\[.*?\]),\s*(\[.*?\]),\s*(\[.*?\]),\s*([\d.]+)\)", sub,
                      flags=re.S)
    gtr = re.search(r'@testset "GTR".*?target = \((\[.*?\]),\s*(\[.*?\]),\s*(\[.*?\]),'
                    r'\s*([\d.]+)\)\s*result = GTR\((\[.*?\]), (\[.*?\])\)', sub, flags=re.S)
    fk = re.search(r'@testset "freeK".*?target = \((\[.*?\]),\s*(\[.*?\]),\s*(\[.*?\]),'
                   r'\s*([\d.]+)\)\s*result = freeK\(\[0.0\], (\[.*?\])\)', sub, flags=re.S)
    sm = re.search(r"setmatrix\((\[.*?\])\)\s*@test result == (\[.*?\])", sub, flags=re.S)

    rates = read("test/likelihood/rates.jl")
    rvecs = [nums(v) for v in re.findall(r"target_vec = \[(.*?)\]", rates)]

    golden = {
        "felsenstein": {
            "primates": {"newick": newicks[0], "logpdf": prim_ll,
                         "source": "test/likelihood/felsenstein.jl:8-20"},
            "simudata": {"newick": newicks[1], "ll": sim_ll, "grad": sim_grad,
                         "source": "test/likelihood/felsenstein.jl:24-40"},
        },
        "multiplephylodist": {"logpdf_factor": 2.0,
                              "source": "test/distributions/phylodist.jl:133-135"},
        "substitution_models": {
            "source": "test/likelihood/substitutionmodels.jl",
            "restriction": {"base_freq": [0.3, 0.7], "U": matrix(restr.group(1)),
                            "D": nums(restr.group(2)), "Uinv": matrix(restr.group(3)),
                            "mu": float(restr.group(4))},
            "jc": {"base_freq": [0.15, 0.45, 0.4], "mu": 1.5,
                   "Q": [[-2 / 3, 1 / 3, 1 / 3], [1 / 3, -2 / 3, 1 / 3], [1 / 3, 1 / 3, -2 / 3]]},
            "gtr": {"U": matrix(gtr.group(1)), "D": nums(gtr.group(2)),
                    "Uinv": matrix(gtr.group(3)), "mu": float(gtr.group(4)),
                    "base_freq": nums(gtr.group(5)), "rates": nums(gtr.group(6))},
            "freek": {"U": matrix(fk.group(1)), "D": nums(fk.group(2)),
                      "Uinv": matrix(fk.group(3)), "mu": float(fk.group(4)),
                      "rates": nums(fk.group(5))},
            "setmatrix": {"input": nums(sm.group(1)), "output": matrix(sm.group(2))},
        },
        "rates": {
            "source": "test/likelihood/rates.jl",
            "alpha": 0.5, "beta": 0.5, "k": 4,
            "mean": rvecs[0], "median": rvecs[1],
            "median_boundaries": rvecs[2], "mean_boundaries": rvecs[3][:3],
        },
    }
    with open(os.path.join(OUT, "golden.json"), "w") as f:
        json.dump(golden, f, indent=1)
    for name in ("primates", "simudata"):
        with open(os.path.join(OUT, f"{name}.json"), "w") as f:
            json.dump(alignment(f"test/likelihood/{name}.nex"), f)
    print("wrote", OUT, file=sys.stderr)


if __name__ == "__main__":
    REF = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MCPHYLO_REFERENCE")
    if not REF or not os.path.isdir(os.path.join(REF, "test", "likelihood")):
        sys.exit("usage: make_golden.py <MCPhylo.jl root> (or set MCPHYLO_REFERENCE)")
    main()

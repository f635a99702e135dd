"""Regenerate the golden fixtures of this directory from the reference checkout.

The reference (PorousMaterials.jl, pure Julia) cannot run here, so its pins are its own
test inputs and known answers: this script copies the input files its tests read
(crystals, force fields, molecules, NIST configurations) into data/ and writes
golden.json with the expected values those tests assert, each with the test file:line.
Run:  python tests/golden/make_fixtures.py path/to/PorousMaterials.jl
"""
import json
import shutil
import sys
from pathlib import Path

if len(sys.argv) != 2:
    sys.exit("usage: python tests/golden/make_fixtures.py path/to/PorousMaterials.jl")
REF = Path(sys.argv[1])
OUT = Path(__file__).resolve().parent / "data"

FILES = {
    "crystals": ["SBMOF-1.cif", "NU-1000_Greg.cif", "zif71_bogus_charges.cif", "test_structure.cif",
                 "LTA.cif", "SOD.cif", "CAXVII_clean.cif", "FIQCEN_clean.cif", "cage_in_space.cif"],
    "forcefields": ["Dreiding.csv", "UFF.csv", "Greg_bogus_ZIF71.csv", "NIST.csv"],
    "molecules": ["Xe", "CO2", "CH4", "CO2EPM2", "X", "He"],
}

GOLDEN = {
    "lennard_jones": {"cite": "test/vdw_energetics.jl:18-21",
                      "cases": [[1.0, 1.0, 3.0, 0.0], [2 ** (2 / 6), 1.0, 3.0, -3.0]]},
    "sbmof1_xe_dreiding": {"cite": "test/vdw_energetics.jl:26-41", "r_cutoff": 12.5,
                           "origin_energy": -5041.58, "point2_cart": [0.494265, 2.22668, 0.450354],
                           "point2_energy": 12945.838, "atol": 0.005},
    "nu1000_ewald": {"cite": "test/electrostatics.jl:12-46", "sr_cutoff": 12.5, "eps": 1e-6,
                     "kreps": [9, 9, 9], "alpha": 0.2471, "alpha_atol": 0.05, "q": 0.8096,
                     "ions": [[[9.535619863743, 20.685576379935, 0.127344239990], 111373.38, 2.5],
                              [[4.269654927228, 23.137319129548, 28.352847101096], -531.0, 0.5],
                              [[-0.047382031804, 7.209555961450, 5.158180463556], -2676.8230141, 0.5]]},
    "required_kreps": {"cite": "test/electrostatics.jl:27-31",
                       "box": [0.5, 0.1, 0.2], "cases": [[2.1, [1, 0, 0]], [5.1, [2, 0, 1]], [10.1, [5, 1, 2]]]},
    "nist_spce": {"cite": "test/electrostatics.jl:48-125", "sr_cutoff": 10.0, "kreps": [5, 5, 5],
                  "alpha_times_L": 5.6, "k2_int_max": 27, "q_H": 0.42380, "rtol": 1e-5,
                  "real": [-5.58889e05, -1.19295e06, -1.96297e06, -3.57226e06],
                  "fourier": [6.27009e03, 6.03495e03, 5.24461e03, 7.58785e03],
                  "self": [-2.84469e06, -5.68938e06, -8.53407e06, -1.42235e07]},
    "zif71_co2": {"cite": "test/electrostatics.jl:130-160", "r_cutoff": 12.8, "es_sr_cutoff": 12.0,
                  "co2_1": [[0.50543, 0.57349, 0.50788], [0.46884, 0.57393, 0.52461], [0.54203, 0.57305, 0.49116]],
                  "co2_2": [[0.50680, 0.38496, 0.50788], [0.54340, 0.38451, 0.49116], [0.47020, 0.38540, 0.52461]],
                  "vdw_1": -132.56, "vdw_atol": 0.01, "es_1": -9.37846564, "es_atol": 0.1,
                  "vdw_both": -311.10392551, "vdw_both_atol": 0.1, "es_both": -36.00, "es_both_atol": 0.3},
    "forcefield_dreiding": {"cite": "test/forcefield.jl:12-30", "sigma_He": 1.0, "epsilon_Zn": 12.0,
                            "sigma2_Zn_He": 4.0, "epsilon_He_Zn": 36.0 ** 0.5, "rep_test_structure": [25, 25, 25]},
    "required_n_pts": {"cite": "test/grid.jl:16-17", "box": [1.0, 10.0, 5.0], "dx": 0.1, "n_pts": [11, 101, 51]},
    "grid_periodic": {"cite": "test/grid.jl:43-55", "crystals": ["LTA.cif", "SOD.cif"], "resolution": 5.0,
                      "cap": 1000.0, "atol": 1e-7},
    "henry_statistical": {"cite": "test/henry.jl:7-34", "insertions_per_volume": 500, "rtol": 0.025,
                          "xe_sbmof1": {"kh_mol_kg_pa": 0.00985348, "u_kj_mol": -39.6811},
                          "co2_caxvii": {"kh_mol_kg_pa": 2.88317e-05, "u_kj_mol": -18.69582223}},
    "nearest_neighbor": {"cite": "test/grid.jl:27-40"},
    "xf_to_id": {"cite": "test/grid.jl:148-177"},
}


# the drop-in functions whose signatures the bindings mirror: (name, reference source file)
DROP_INS = [("henry_coefficient", "src/henry.jl"), ("energy_grid", "src/grid.jl")]


def _signature(path: Path, name: str) -> dict:
    """Positional argument and keyword names of `function name(...)` in a reference source file,
    with the file:line range of the signature."""
    import re

    lines = path.read_text().splitlines()
    start = next(i for i, ln in enumerate(lines) if re.match(rf"\s*function {name}\(", ln))
    text, depth, end = "", 0, start
    for end in range(start, len(lines)):
        for ch in lines[end]:
            if ch == "(":
                depth += 1
            elif ch == ")":
                depth -= 1
            text += ch
            if depth == 0 and text.count("(") > 0:
                break
        if depth == 0 and "(" in text:
            break
        text += " "
    inner = text[text.index("(") + 1:text.rindex(")")]
    pos, _, kw = inner.partition(";")

    def names(part):
        out, depth, cur = [], 0, ""
        for ch in part + ",":
            if ch in "({[":
                depth += 1
            elif ch in ")}]":
                depth -= 1
            if ch == "," and depth == 0:
                if cur.strip():
                    out.append(re.match(r"\s*([A-Za-z_][A-Za-z_0-9!²]*)", cur).group(1))
                cur = ""
            else:
                cur += ch
        return out

    rel = path.relative_to(REF)
    return {"cite": f"{rel}:{start + 1}-{end + 1}", "positional": names(pos), "keywords": names(kw)}


def main():
    OUT.mkdir(parents=True, exist_ok=True)
    GOLDEN["drop_in_signatures"] = {name: _signature(REF / src, name) for name, src in DROP_INS}
    td = REF / "test" / "data"
    for sub, names in FILES.items():
        (OUT / sub).mkdir(exist_ok=True)
        for n in names:
            src = td / sub / n
            if src.is_dir():
                dst = OUT / sub / n
                dst.mkdir(exist_ok=True)
                for f in src.iterdir():
                    shutil.copy(f, dst / f.name)
            else:
                shutil.copy(src, OUT / sub / n)
    shutil.copy(td / "atomicmasses.csv", OUT / "atomicmasses.csv")
    (OUT / "nist").mkdir(exist_ok=True)
    for c in range(1, 5):
        shutil.copy(REF / "test" / "nist" / "electrostatics" / f"spce_sample_config_periodic{c}.txt",
                    OUT / "nist" / f"spce_sample_config_periodic{c}.txt")
    (Path(__file__).resolve().parent / "golden.json").write_text(json.dumps(GOLDEN, indent=1))


if __name__ == "__main__":
    main()

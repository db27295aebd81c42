"""Generate the golden fixtures under tests/golden/ from the reference's own test data.

Reads the reference's test/data/{param.in, mat.in, system.in, TempDis.dat} (a 25x25x1 Fourier
run of 10 steps whose final Temp_p the reference wrote with final_print) and stores them in
tempdis_25x25.json: the three input decks verbatim (they are the run's inputs) and the 625
golden temperatures.  Also stores test/data/tempdep.in (the reference's temperature-table
format: T, kappa, rho, c per row) verbatim in tempdep_table.json.  Run from the repository root with the reference's checkout as argument:

    python tests/golden/make_golden.py <path to the HeatFlow checkout>
"""
import json
import os
import sys


def main(ref_root: str):
    data = os.path.join(ref_root, "test", "data")
    rd = lambda n: open(os.path.join(data, n)).read()
    vals = [float(t) for t in rd("TempDis.dat").split()]
    out = {
        "source": "reference test/data: param.in, mat.in, system.in, TempDis.dat",
        "param_in": rd("param.in"),
        "mat_in": rd("mat.in"),
        "system_in": rd("system.in"),
        "ntime": 10,
        "tempdis": vals,
        "print_precision": "ES16.8",
    }
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(here, "tempdis_25x25.json"), "w") as f:
        json.dump(out, f, indent=1)
    print(f"wrote {len(vals)} golden values")
    with open(os.path.join(here, "tempdep_table.json"), "w") as f:
        json.dump({"source": "reference test/data/tempdep.in", "text": rd("tempdep.in")}, f, indent=1)
    print("wrote the temperature table")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path to the HeatFlow checkout>")
    main(sys.argv[1])

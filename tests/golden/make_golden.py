"""Regenerates the golden fixtures under tests/golden/ from the reference's own run artefacts.

Run once in a container where the reference checkout is mounted:

    python tests/golden/make_golden.py REFERENCE_DIR

It copies the input deck of the reference's `try/` run (a 27 445-step run of the
Filled_Channel deck: 300 brush chains x 10 beads + 3000 solvent beads, box 30x20x40) and
extracts the known-answer values that the reference printed in try/log and try/mfa_output:

* the LJ cut-off and shift tables (init_params.f90:742-761 print them),
* the total shifted-LJ energy of try/conf_old (check_fluid_fluid, util.f90:284-330),
* the first centre-of-mass velocity (init_config.f90:336-343),
* the BIN_TYPE 0 binning boxes (make_binning_boxes.f90, written to mfa_output).

The try/ run was built with the flags of inputs/Filled_Channel/control_simulation.h (the log's
banner lines match it: BIN_TYPE 0, SOLVENT 3, BRUSH_IN_GOOD_SV, WALL 2, DPD_CUT_OFF 2.24,
BENDING, ORIENTATION, FORCE_SWITCH_ON, PROFILES), so that header is copied beside the deck.
Nothing at test time reads the reference checkout.
"""
import gzip
import json
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def _floats(line):
    return [float(x) for x in re.findall(r"-?\d+\.\d+(?:[eE][-+]?\d+)?", line)]


def main(ref):
    out = os.path.join(HERE, "try")
    os.makedirs(out, exist_ok=True)
    for name in ("system_input", "mfa_input"):
        shutil.copyfile(os.path.join(ref, "try", name), os.path.join(out, name))
    shutil.copyfile(os.path.join(ref, "inputs", "Filled_Channel", "control_simulation.h"),
                    os.path.join(out, "control_simulation.h"))
    # conf_old: the start of the run; conf_new: the restart file that the run wrote
    # (store_config.f90:14-63), the byte-level fixture of the conf_new writer
    for name in ("conf_old", "conf_new"):
        with open(os.path.join(ref, "try", name), "rb") as f, \
                gzip.GzipFile(os.path.join(out, name + ".gz"), "wb", mtime=0) as g:
            g.write(f.read())

    kat = {"cutoffs": [], "shifts": []}
    with open(os.path.join(ref, "try", "log")) as f:
        for line in f:
            if "interacts with cutoffs" in line:
                kat["cutoffs"].append(_floats(line.split(":", 1)[1]))
            elif "potential's shifts" in line:
                kat["shifts"].append(_floats(line.split(":", 1)[1]))
            elif "[check_fluid_fluid]" in line:
                kat["v_fluid_fluid_check"] = _floats(line)[0]
            elif "V_fluid_fluid for the first configuration" in line:
                kat["v_fluid_fluid_f16_5"] = _floats(line)[0]
            elif "First Vcm=" in line:
                kat["first_vcm"] = _floats(line)
            elif "Maximum cut-off radius for potentials" in line:
                kat["r_cut_max_potentials"] = _floats(line)[0]
            elif "DPD cut-off radius" in line:
                kat["r_cut_dpd"] = _floats(line)[0]
            elif "Max  cut-off radius for ALL" in line:
                kat["r_cut_max"] = _floats(line)[0]
            elif "Skin for verlet lists" in line:
                kat["skin"] = _floats(line)[0]
    with open(os.path.join(ref, "try", "mfa_output")) as f:
        lines = f.read().splitlines()
    for i, line in enumerate(lines):
        if line.strip().endswith("binning boxes"):
            kat["binning_boxes"] = [int(x) for x in line.split()[:3]]
        if line.strip().endswith("binning distances"):
            kat["binning_distances"] = [float(x) for x in line.split()[:3]]
    with open(os.path.join(out, "kat.json"), "w") as f:
        json.dump(kat, f, indent=1, sort_keys=True)
    print(json.dumps(kat, indent=1, sort_keys=True))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py REFERENCE_DIR")
    main(sys.argv[1])

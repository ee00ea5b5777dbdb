"""Generate tests/golden/ fixtures from QDng's own test inputs and goldens.

Run here (where the QDng source tree is mounted) with
    python tests/golden/make_fixtures.py /root/reference
It reads the raw-binary .op/.wf fixtures with their .meta grids from the
reference's tests/ directory (FileSingle raw format: little-endian float64 /
complex128, src/tools/FileSingle.h:1243-1290) and the expected output lines
of tests/checktests.sh, and writes
    qdng_fixtures.npz        -- the arrays
    checktests_golden.json   -- the expected values, parsed to numbers
Neither file is read from the reference at test time.
"""
import json
import os
import re
import sys

import numpy as np


def read_meta(path):
    meta = {}
    for line in open(path):
        line = line.strip()
        if not line or line.startswith("#") or "=" not in line:
            continue
        k, v = line.split("=", 1)
        meta[k.strip()] = v.strip()
    return meta


def main(ref):
    tdir = os.path.join(ref, "tests")
    out = {}
    for name in ["GridPot0", "GridPot1", "GridDip0", "GridDip01", "GridGM_00"]:
        meta = read_meta(os.path.join(tdir, name + ".meta"))
        n = int(meta["N0"])
        out[name] = np.fromfile(os.path.join(tdir, name + ".op"), dtype="<f8")[:n]
        out[name + "_grid"] = np.array([n, float(meta["xmin0"]), float(meta["xmax0"])])
    for name in ["GridGauss", "GridPot0_ef_0", "GridPot0_ef_1", "GridPot0_ef_2", "GridPot0_ef_3"]:
        meta_name = "GridPot0_ef" if name.startswith("GridPot0_ef") else name
        meta = read_meta(os.path.join(tdir, meta_name + ".meta"))
        n = int(meta["N0"])
        out[name] = np.fromfile(os.path.join(tdir, name + ".wf"), dtype="<c16")[:n]
    for name in ["GridLaser_w0.00713", "GridLaser_w0.176"]:
        meta = read_meta(os.path.join(tdir, name + ".meta"))
        nt = int(meta["Nt"])
        key = name.replace(".", "p")
        out[key] = np.fromfile(os.path.join(tdir, name + ".op"), dtype="<f8")[:nt]
        out[key + "_dt"] = np.array([float(meta["dt"])])
    here = os.path.dirname(os.path.abspath(__file__))
    np.savez_compressed(os.path.join(here, "qdng_fixtures.npz"), **out)

    text = open(os.path.join(tdir, "checktests.sh")).read()
    gold = {"propagation": {}, "expec": {}, "tge_imag": [], "tge_ac": [], "tge_initial": None}

    def nums(s):
        vals = []
        for tok in s.split():
            if "," in tok and tok.endswith("i"):
                re_, im = tok[:-1].split(",")
                vals.append([float(re_), float(im)])
            else:
                vals.append(float(tok.replace("[0-9]*", "").replace("[0-9]", "")))
        return vals

    for m in re.finditer(r'^CheckT (\S+)\s+"([^"]+)"', text, flags=re.M):
        gold["propagation"][m.group(1)] = {"text": m.group(2), "values": nums(m.group(2))}
    for m in re.finditer(r'^CheckT-Expec (\S+)\s+"([^"]+)"', text, flags=re.M):
        gold["expec"][m.group(1)] = {"text": m.group(2), "values": nums(m.group(2))}
    im = re.search(r"CheckTGE-im-Energy\(\)\n\{(.*?)\n\}", text, flags=re.S).group(1)
    gold["tge_imag"] = [[int(a), b] for a, b in re.findall(r"grep '(\d)\[\[:space:\]\]\*([0-9.]+)'", im)]
    ac = re.search(r"CheckTGE-ac-Energy\(\)\n\{(.*?)\n\}", text, flags=re.S).group(1)
    gold["tge_ac"] = [[int(a), b] for a, b in re.findall(r"grep '(\d)\[\[:space:\]\]\*([0-9.]+)'", ac)]
    m = re.search(r"Initial Norm & energy: ([0-9.e+-]+)\.\*([0-9.e+-]+)", text)
    gold["tge_initial"] = [m.group(1), m.group(2)]
    json.dump(gold, open(os.path.join(here, "checktests_golden.json"), "w"), indent=1)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")

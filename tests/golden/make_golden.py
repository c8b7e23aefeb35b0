"""Regenerates the golden fixtures in this folder from the reference checkout.

The reference's own tests hold the only golden vectors for the GAP path
(SOAP vectors, SOAP gradients, distance_2b energies/forces, small-cell energies).
This script copies those data files verbatim, and extracts the arrays that the
reference keeps inline in its test sources, into small files that travel with
the repository.  It reads the reference checkout named by the environment variable
QUIP_REFERENCE (required) and is only run by hand; tests never read the reference at
run time:  QUIP_REFERENCE=<path to the QUIP checkout> python tests/golden/make_golden.py

Sources:
  tests/Si.np1.xyz, tests/Si.soap.cur_points.json       (test_gapfit.py:93-95, :58)
  tests/test_descriptor.py:39-190                          (C2H SOAP gradients)
  tests/GAP.xml, tests/GAP.xml.sparseX.*, gap_sample.xyz  (test_gappot.py:30-48)
  tests/test_potential_cell.py:31-43                       (energies in small cells)
  tests/Si.two_descriptors.json                            (distance_2b + SOAP sparse points)
"""
import ast
import glob
import json
import os
import shutil
import sys

import numpy as np

REF = os.environ.get("QUIP_REFERENCE")
OUT = os.path.dirname(os.path.abspath(__file__))


def main():
    if not REF or not os.path.isdir(os.path.join(REF, "tests")):
        sys.exit("set QUIP_REFERENCE to the QUIP checkout (the folder that holds tests/)")
    t = os.path.join(REF, "tests")
    shutil.copy(os.path.join(t, "Si.np1.xyz"), os.path.join(OUT, "Si.np1.xyz"))
    d = json.load(open(os.path.join(t, "Si.soap.cur_points.json")))
    c = d["coords"][0]
    np.savez_compressed(os.path.join(OUT, "si_soap_cur_points.npz"),
                        sparsex=np.array(c["sparsex"]).reshape(-1, c["dimensions"]),
                        alpha=np.array(c["alpha"]), cutoff=np.array(c["cutoff"]),
                        index=np.array(d["index"][0]), config=np.array(d["config"]))
    d2 = json.load(open(os.path.join(t, "Si.two_descriptors.json")))
    np.savez_compressed(os.path.join(OUT, "si_two_descriptors.npz"),
                        d2b_sparsex=np.array(d2["coords"][0]["sparsex"]),
                        d2b_index=np.array(d2["index"][0]),
                        soap_sparsex=np.array(d2["coords"][1]["sparsex"]).reshape(-1, d2["coords"][1]["dimensions"]),
                        soap_index=np.array(d2["index"][1]), config=np.array(d2["config"]))
    # C2H descriptor gradients: arrays live inline in the test source
    src = open(os.path.join(t, "test_descriptor.py")).read()
    tree = ast.parse(src)
    found = {}
    for node in ast.walk(tree):
        if isinstance(node, ast.Assign) and isinstance(node.targets[0], ast.Attribute):
            name = node.targets[0].attr
            if name in ("ref_grad_index_0based", "ref_grad_array") and isinstance(node.value, ast.Call):
                found[name] = np.array(ast.literal_eval(node.value.args[0]))
    np.savez_compressed(os.path.join(OUT, "c2h_soap_grad.npz"), grad=found["ref_grad_array"],
                        grad_index=found["ref_grad_index_0based"])
    wd = os.path.join(OUT, "gap_water")
    os.makedirs(wd, exist_ok=True)
    for f in ["GAP.xml", "gap_sample.xyz"] + [os.path.basename(p) for p in glob.glob(os.path.join(t, "GAP.xml.sparseX.*"))]:
        shutil.copy(os.path.join(t, f), os.path.join(wd, f))
    # small-cell energies (test_potential_cell.py): cell sizes and reference energies
    src = open(os.path.join(t, "test_potential_cell.py")).read()
    tree = ast.parse(src)
    energies = None
    for node in ast.walk(tree):
        if isinstance(node, ast.Assign) and isinstance(node.targets[0], ast.Attribute) and node.targets[0].attr == "ref_energies":
            energies = ast.literal_eval(node.value)
    json.dump({"cell_sizes": list(np.linspace(2.5, 4.5, 5)), "positions": [[0., 0., 0.], [1., 1., 1.]],
               "symbols": "HH", "ref_energies": energies, "tol": 1e-6},
              open(os.path.join(OUT, "potential_cell.json"), "w"), indent=1)
    print("golden fixtures written to", OUT)


if __name__ == "__main__":
    sys.exit(main())

"""Writes tests/golden/eps_reference.json.gz: the reference's own neighbour
threshold and its two- and three-hop bounds for a grid of thresholds and
length pairs, printed by oracle/_ref/ref_eps (built by oracle/build_ref.py from
the reference's cuda/SpecialFunctors.hcu).  Run where the reference tree is
present:

    IDB_REFERENCE_TREE=<reference checkout> python tests/golden/make_eps_golden.py
"""
import gzip
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import build_ref  # noqa: E402

if not build_ref.build():
    sys.exit("IDB_REFERENCE_TREE does not name a reference tree")
exe = build_ref.EPS_EXE
out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
table = json.loads(out)
table["source"] = ("epsilonOneFunctorClass<false> and <true> (cuda/SpecialFunctors.hcu:245-274), "
                   "epsilonTwoFunctorClass and epsilonThreeFunctorClass <false> and <true> "
                   "(:276-344), compiled on the host by oracle/build_ref.py")
path = os.path.join(HERE, "eps_reference.json.gz")
with gzip.open(path, "wt") as f:
    json.dump(table, f, separators=(",", ":"))
print("wrote", path)

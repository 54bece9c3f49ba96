"""Extract the reference data the package ships: SuperFast (superfast.esm) and the 72-level
hybrid sigma-pressure table (hybrid_coefs_L72.json).

The reference mounts SuperFast by ``$ref`` to a sibling checkout that is not vendored
(``reseact.esm:12714-12716``); its only in-tree copy is the inline reaction system of
``prototypes/g2_depsink/g2_nodep.esm`` (species ``:1781``, parameters ``:402``, reactions
``:450-1780``, template ``:1861``, golden tests ``:9-400``).  The mechanism is data the
drop-in must share with the reference, so this script copies that reaction system (schema
unchanged, prose descriptions dropped) for use where the reference tree is absent.

The 72-level table is ``prototypes/reseact_3d_chem/hybrid_coefs_L72.json`` (dA, dB, Ap, Bp).

    python reseact/esm_gb300/mechanisms/extract_reference_data.py REFERENCE_CHECKOUT

REFERENCE_CHECKOUT is the root of an EarthSciML/reseact.esm checkout (required).
"""
import json
import os
import sys

if len(sys.argv) != 2:
    sys.exit("usage: extract_reference_data.py REFERENCE_CHECKOUT")
ref = sys.argv[1]
src = os.path.join(ref, "prototypes", "g2_depsink", "g2_nodep.esm")
with open(src) as fh:
    doc = json.load(fh)
rs = doc["reaction_systems"]["SuperFast"]
keep = {k: rs[k] for k in ("parameters", "species", "reactions", "expression_templates", "tests")}
for t in keep["tests"]:
    t.pop("description", None)
for v in list(keep["species"].values()) + list(keep["parameters"].values()):
    v.pop("description", None)
out = {"esm": doc.get("esm", "1.0.0"),
       "metadata": {"name": "SuperFast",
                    "source": "prototypes/g2_depsink/g2_nodep.esm reaction_systems.SuperFast"},
       "reaction_systems": {"SuperFast": keep}}
dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "superfast.esm")
with open(dst, "w") as fh:
    json.dump(out, fh, indent=1)
print("wrote", dst)

hsrc = os.path.join(ref, "prototypes", "reseact_3d_chem", "hybrid_coefs_L72.json")
with open(hsrc) as fh:
    h = json.load(fh)
hdst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "hybrid_coefs_L72.json")
with open(hdst, "w") as fh:
    json.dump({k: h[k] for k in ("dA", "dB", "Ap", "Bp")}, fh)
print("wrote", hdst)

"""Generate ``tests/golden/tables_ref.json`` from the reference's shipped tables.

Run in a checkout where the reference tree is mounted, given by ``--ref`` or
the ``CTR_REFERENCE_ROOT`` environment variable (no default).  It parses every
``include/constants_*.h`` of the reference and records, for each array, its
declared shape and the SHA-256 of its value tokens exactly as printed in the
header (``%d`` / ``%+3.2f``, signed zeros kept), joined by commas.  Only the
digests and shapes are committed; the tests regenerate the tables with the
oracle's and the library's own generators and compare digests.
"""

import argparse
import glob
import hashlib
import json
import os
import re


def parse_header(path):
    txt = open(path).read()
    out = {}
    for m in re.finditer(r"static\s+(short int|float)\s+(\w+)((?:\[\d+\])+)\s*=\s*\{([^}]*)\}", txt):
        typ, name, dims, body = m.groups()
        dims = [int(d) for d in re.findall(r"\[(\d+)\]", dims)]
        toks = [t.strip() for t in body.split(",") if t.strip()]
        n = 1
        for d in dims:
            n *= d
        if len(toks) != n:
            raise ValueError("%s: %d values for shape %s" % (name, len(toks), dims))
        out[name] = {"shape": dims, "type": typ, "tokens": toks}
    return out


def digest(tokens):
    return hashlib.sha256(",".join(tokens).encode()).hexdigest()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("CTR_REFERENCE_ROOT"), required="CTR_REFERENCE_ROOT" not in os.environ)
    ap.add_argument("--out", default=os.path.join(os.path.dirname(__file__), "tables_ref.json"))
    args = ap.parse_args()
    res = {}
    for f in sorted(glob.glob(os.path.join(args.ref, "include", "constants_*.h"))):
        for name, t in parse_header(f).items():
            res[name] = {
                "header": "include/" + os.path.basename(f),
                "shape": t["shape"],
                "type": t["type"],
                "sha256": digest(t["tokens"]),
            }
    with open(args.out, "w") as fh:
        json.dump(res, fh, indent=1, sort_keys=True)
    print("wrote %d tables to %s" % (len(res), args.out))


if __name__ == "__main__":
    main()

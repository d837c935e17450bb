"""Import pattern -> nanokernel mapping files from a checkout of the reference project.

Usage: python tests/golden/import_mappings.py <reference root>   (or SPREG_REFERENCE=<root>)

Copies sbench/SOP/mappings/mapping_<id>.txt and sbench/SOP/identity_mappings/*/mapping_<id>.txt
into the package's mapping directory (sparse-register-tiling_gb300/spreg/mappings) after checking that each file's id equals md5(str({pattern: list}))[-5:]
of its content, the rule by which the reference names them (sbench/SOP/mapping.py:9).  The
files are data tables of the reference's interface: a mapping id only means the same
nanokernel set if the content is byte-for-byte the same, so they are carried over unchanged.
"""
from __future__ import annotations

import ast
import glob
import hashlib
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
DEST = os.path.join(os.path.dirname(os.path.dirname(HERE)), "sparse-register-tiling_gb300", "spreg", "mappings")


def content_id(text: str) -> str:
    lines = [ln for ln in text.splitlines() if ln.strip()]
    d = {}
    for ln in lines[1:]:
        k, v = ln.split(":", 1)
        d[int(k)] = ast.literal_eval(v.strip())
    return hashlib.md5(str(d).encode("utf-8")).hexdigest()[-5:]


def main(root: str) -> int:
    pats = [os.path.join(root, "sbench/SOP/mappings/mapping_*.txt"),
            os.path.join(root, "sbench/SOP/identity_mappings/*/mapping_*.txt")]
    n = 0
    for pat in pats:
        for path in sorted(glob.glob(pat)):
            name = os.path.basename(path)
            text = open(path).read()
            cid = content_id(text)
            if cid != name[len("mapping_"):-len(".txt")]:
                print(f"skip {path}: content id {cid} != file id", file=sys.stderr)
                continue
            with open(os.path.join(DEST, name), "w") as f:
                f.write(text)
            n += 1
    print(f"imported {n} mappings into {DEST}")
    return 0


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SPREG_REFERENCE")
    if not root:
        sys.exit("usage: import_mappings.py <reference root> (or set SPREG_REFERENCE)")
    sys.exit(main(root))

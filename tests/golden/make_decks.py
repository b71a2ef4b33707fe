"""Copy the reference's own control files (its `input/` directory) into
tests/golden/decks/ as test inputs, byte for byte.

    python tests/golden/make_decks.py [REFERENCE_ROOT]

The decks are BookLeaf's input data (Crown Copyright 2018 AWE, GPL-3.0 or
later, as the rest of BookLeaf); they travel with the tests so that the GPU
tests can run them where the reference tree is absent.
"""
import hashlib
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "decks")


def main(root):
    src = os.path.join(root, "input")
    os.makedirs(OUT, exist_ok=True)
    for name in sorted(os.listdir(src)):
        path = os.path.join(src, name)
        if not os.path.isfile(path):
            continue
        shutil.copyfile(path, os.path.join(OUT, name))
        with open(path, "rb") as f:
            print(name, hashlib.sha256(f.read()).hexdigest()[:16])


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")

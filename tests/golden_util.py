"""Loads the reference-generated fixtures in tests/golden/ (see make_golden.py)."""
import glob
import hashlib
import os
import re

import numpy as np

import graphgen

GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def names():
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN_DIR, "*.npz")))


class Fixture:
    def __init__(self, name):
        z = np.load(os.path.join(GOLDEN_DIR, name + ".npz"))
        self.name = name
        self.z = z
        self.V = int(z["V"])
        self.root = int(z["root"])
        kind, a, b, seed = [str(x) for x in z["gen"]]
        if kind == "rmat":
            self.src, self.dst, self.w = graphgen.rmat(int(a), int(b), int(seed), weighted=True)
        elif kind == "grid":
            self.src, self.dst, self.w = graphgen.grid(int(a), seed=int(seed), weighted=True)
        else:
            self.src, self.dst, self.w = z["src"], z["dst"], z["w"]
        rec = graphgen.to_records(self.src, self.dst, self.w)
        if name == "edgecase":
            rec += b"\x01\x02\x03\x04\x05"
        if hashlib.sha256(rec).hexdigest() != str(z["edges_sha256"]):
            raise AssertionError(f"{name}: regenerated edges differ from the fixture's")

    def __getitem__(self, k):
        return self.z[k]

    def stdout(self, app):
        return str(self.z[app + "_stdout"])

    def summary(self, app):
        return str(self.z[app + "_summary"])

    def printed_active(self, app):
        """The `active(i)>=n` values the reference printed (forward pass for bc)."""
        return [int(m) for m in re.findall(r"active\(\d+\)>=(\d+)", self.stdout(app))]

    def printed_deltas(self):
        return [float(m) for m in re.findall(r"delta\(\d+\)=([0-9.]+)", self.stdout("pr"))]

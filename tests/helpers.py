"""Shared helpers for the parity tests."""
import hashlib
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_golden(name):
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        return json.load(f)


def golden_arrays(g):
    mean, unc = [], []
    for est in g["estimators"]:
        for m, u in est:
            mean.append(float.fromhex(m) if "x" in m else float(m))
            unc.append(float.fromhex(u) if "x" in u else float(u))
    return np.array(mean), np.array(unc)


def bits(a):
    return np.ascontiguousarray(np.asarray(a, np.float64)).view(np.uint64)


def digest_sha(d):
    return hashlib.sha256(np.ascontiguousarray(d, np.uint64).tobytes()).hexdigest()


def same_bits(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    if a.shape != b.shape:
        return False
    return bool(np.all((bits(a) == bits(b)) | (np.isnan(a) & np.isnan(b))))

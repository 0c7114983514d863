"""Loader for tests/golden/bgpq_ref_cases.npz (made by tests/golden/make_golden.py
from the reference's own heap headers)."""
import json
import os

import numpy as np

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bgpq_ref_cases.npz")
_data = None


def data():
    global _data
    if _data is None:
        _data = np.load(PATH)
    return _data


def meta():
    return json.loads(bytes(data()["meta"]).decode())


def case(i):
    d = data()
    p = f"c{i}_"
    out = {k[len(p):]: d[k] for k in d.files if k.startswith(p)}
    out.update(meta()[i])
    return out

"""Loader for the golden vectors made by tests/golden/make_golden.py from the
reference's own heap headers: `small` (bgpq_ref_cases.npz, batch 16-64) and
`large` (bgpq_ref_cases_large.npz, batch 256-2048); and the insert/retrieve
sequences of the reference's retrieving heap (retrieve_ref_cases.npz)."""
import json
import os

import numpy as np

_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FILES = {"small": "bgpq_ref_cases.npz", "large": "bgpq_ref_cases_large.npz"}
PATH = os.path.join(_DIR, FILES["small"])
_data = {}


def data(which="small"):
    if which not in _data:
        _data[which] = np.load(os.path.join(_DIR, FILES[which]))
    return _data[which]


def meta(which="small"):
    return json.loads(bytes(data(which)["meta"]).decode())


def case(i, which="small"):
    d = data(which)
    p = f"c{i}_"
    out = {k[len(p):]: d[k] for k in d.files if k.startswith(p)}
    out.update(meta(which)[i])
    return out


def all_ids():
    """(set, index) of every golden case, for parametrising."""
    return [(w, i) for w in FILES for i in range(len(meta(w)))]


RETRIEVE_FILE = "retrieve_ref_cases.npz"


def retrieve_meta():
    return json.loads(bytes(_retrieve_data()["meta"]).decode())


def _retrieve_data():
    if "retrieve" not in _data:
        _data["retrieve"] = np.load(os.path.join(_DIR, RETRIEVE_FILE))
    return _data["retrieve"]


def retrieve_case(i):
    """ops (positive: insert that many of `keys` in order; negative: retrieve
    -op keys), taken (each retrieve's count), runs (retrieved keys, joined),
    final_nodes / final_pb / final_counters (the reference heap's valid nodes,
    valid partial buffer and {batch count, pb size} after the sequence), and
    the meta fields (key, batch_size, batch_num, seed, ties)."""
    d = _retrieve_data()
    p = f"c{i}_"
    out = {k[len(p):]: d[k] for k in d.files if k.startswith(p)}
    out.update(retrieve_meta()[i])
    return out

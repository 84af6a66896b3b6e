"""Loads a PDM fast-expectation fixture (tests/golden/*_npdm.npz)."""
import json
import os

import numpy as np

from conftest import GOLDEN
from b2g.capi import PairSeq
from b2g.problem import PAIR_FIELDS

LAYOUT = ("p_off", "p_trans", "p_nblk", "b_off", "b_rows", "b_cols")
TERMS = ("t_k", "t_part", "t_roff", "t_rsize", "t_f")


def load(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = {k: z[k] for k in z.files if k != "meta"}
    d["meta"] = json.loads(str(z["meta"]))
    d["seq"] = PairSeq({k: d[k] for k in PAIR_FIELDS})
    d["layout"] = {k: d[k] for k in LAYOUT}
    d["terms"] = {k: d[k] for k in TERMS}
    return d

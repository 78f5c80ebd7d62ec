"""Loader for the reference golden fixtures (tests/golden/reference_kernels.npz)."""
import os
from collections import defaultdict

import numpy as np

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "reference_kernels.npz")


def load(family=None):
    data = np.load(PATH, allow_pickle=False)
    cases = defaultdict(dict)
    for key in data.files:
        fam, idx, name = key.split("/")
        if family is None or fam == family:
            cases[(fam, idx)][name] = data[key]
    out = []
    for (fam, idx), c in sorted(cases.items()):
        c = {k: (v.item() if v.ndim == 0 and v.dtype.kind in "iubU" else v) for k, v in c.items()}
        c["family"], c["id"] = fam, f"{fam}-{idx}"
        out.append(c)
    return out

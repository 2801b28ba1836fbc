"""Loading helpers for the golden fixtures in tests/golden/."""
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def case_names():
    import lbcases
    return [b().name for b in lbcases.CASES]


def load(name):
    g = np.load(os.path.join(GOLDEN, name + ".npz"))
    meta = json.loads(str(g["meta"]))
    return g, meta


def load_fingerprint(name):
    with open(os.path.join(GOLDEN, name + ".json")) as f:
        return json.load(f)


def stats_close(a, b, rtol=1e-12, atol=1e-14):
    """Reductions are sums in a different order than the reference: compare to
    rounding of the summation, not bit for bit."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return np.all(np.abs(a - b) <= atol + rtol * np.abs(b)), np.max(np.abs(a - b) / (atol + np.abs(b)))

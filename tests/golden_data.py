"""Loader of the SEAL-generated fixture tests/golden/ckks_n4096.npz."""
from pathlib import Path

import numpy as np

PATH = Path(__file__).parent / "golden" / "ckks_n4096.npz"


def load():
    d = np.load(PATH)
    return {k: d[k] for k in d.files}

"""Benchmark models used by the tests (the presets live in the library package)."""
import os
import sys

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "heom-quick2_gb300"))
from heomq.models import siam, dqd, hund, iv_sweep, SIAM_L3, DQD_L4, HUND_L2  # noqa: E402,F401

CFG0, CFG1, CFG4 = SIAM_L3, DQD_L4, HUND_L2


def prony_table():
    """A Prony table (psfjob) that is not a restatement of a Pade decomposition: the Pade table
    of a T = 0.3 band with its poles stretched by 1.15 and its residues rotated by 0.2 rad."""
    import numpy as np
    import heomq

    t = heomq.psf_table_from_pade(1, 10.0, 0.3, tpsf=2.0)
    return dict(t, pole=t["pole"] * 1.15, coef=t["coef"] * np.exp(0.2j))

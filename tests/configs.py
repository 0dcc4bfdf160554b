"""Benchmark models used by the tests (the presets live in the library package)."""
import os
import sys

sys.path.insert(0, os.path.join(os.path.dirname(os.path.abspath(__file__)), "..", "heom-quick2_gb300"))
from heomq.models import siam, dqd, hund, iv_sweep, SIAM_L3, DQD_L4, HUND_L2  # noqa: E402,F401

CFG0, CFG1, CFG4 = SIAM_L3, DQD_L4, HUND_L2

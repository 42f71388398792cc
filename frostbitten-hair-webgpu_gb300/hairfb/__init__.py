"""hairfb -- GB300-native hair hot path (host side).

Python mirror of the reference's per-pass operator interface
(src/passes/*/<Pass>.ts) over the C-ABI of ``libhairfb.so``.
"""
from .config import HairConfig, HfbConfig, SimulationParams  # noqa: F401

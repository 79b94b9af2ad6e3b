"""ctypes declarations of the side entry points added after the base set (voxel, MLP, batch)."""
from __future__ import annotations

import ctypes as C


def declare(L: C.CDLL) -> None:
    """Declares argtypes for optional entry points present in this build."""
    return None

"""GB300-native (sm_103a) implementation of QPAD's per-xi-slice quasi-static loop.

The compute path is CUDA built into ``qpad_gb300/_lib/libqpad_gpu.so`` behind the C ABI in
``include/qpad_gpu.h``; ``api`` mirrors the reference's Fortran call surface over it.
"""
from . import _capi, api, decks  # noqa: F401
from .api import (Batch, Beam3D, Field, QpadError, Simulation, SliceStats, Species2D, add_f1,  # noqa: F401
                  add_f1_dim, load_beam, load_plasma)
from .runner import build_simulation, deck_inputs  # noqa: F401

__all__ = ["Simulation", "Batch", "Species2D", "Beam3D", "Field", "QpadError", "SliceStats", "add_f1", "add_f1_dim",
           "load_plasma", "load_beam", "build_simulation", "deck_inputs", "decks"]

"""GB300-native fused collide-and-stream pull step of metaLBM.

Host-side mirror of the reference's template surface for this hot path:
``InputDeck`` carries the Input.in parameters (src/Input_prod.in:16-53) that
select Lattice / Collision / ForcingScheme / Force; ``Lattice`` owns one
periodic lattice on one GPU through the C ABI (include/mlbm/mlbm.h);
``Algorithm`` keeps metaLBM's Algorithm interface (iterate / pack / unpack /
isStored, Algorithm.h:23-29, 132-147, 326-358) on top of it.
"""
from .capi import MlbmError
from .lattice import Algorithm, InputDeck, Lattice, MlpModel

__all__ = ["Algorithm", "InputDeck", "Lattice", "MlbmError", "MlpModel"]

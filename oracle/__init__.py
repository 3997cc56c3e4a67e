"""Test oracle for the fused collide-and-stream pull step.

TEST INFRASTRUCTURE ONLY. Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg may import this package, and only as the checker or as the
timed CPU baseline; the product library (metalbm_gb300) never does.

* ``OraclePort`` wraps the C restatement in oracle/mlbm_oracle.c (built into
  oracle/_build/liboracle.so by ``build_port``).
* ``run_reference`` runs a reference metaLBM binary built by
  oracle/build_ref.py (only where the reference sources exist).
"""
from .port import (ALPHA_REFERENCE, ALPHA_RESIDUAL, GUESS_PREVIOUS, GUESS_TWO, OraclePort,
                   OracleConfig, build_port, lattice_tables)

__all__ = ["ALPHA_REFERENCE", "ALPHA_RESIDUAL", "GUESS_PREVIOUS", "GUESS_TWO", "OraclePort",
           "OracleConfig", "build_port", "lattice_tables"]

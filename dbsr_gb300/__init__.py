"""GB300 (sm_103a) Hamiltonian-block assembly for DBSR_MAT3.

``dbsr_gb300.api.Assembler`` is the host-side mirror of the reference's
Gen_matrix interface on top of the C ABI in ``include/dbsrg.h``
(``dbsr_gb300/_build/libdbsrgpu.so``); ``dbsr_gb300.synth`` generates the
seeded benchmark workloads.
"""
from .api import FACTOR_FP64, PLAIN_FP64, RK, SK, SPLIT_BF16, Assembler  # noqa: F401
from ._lib import DbsrgError  # noqa: F401

__all__ = ["Assembler", "DbsrgError", "PLAIN_FP64", "SPLIT_BF16", "FACTOR_FP64", "RK", "SK"]

"""CPU oracle of the reionization grid step — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU baseline import this
package; the product library never does.  `OracleBackend` wraps the plain-C
restatement (oracle/mx_oracle.c, built into oracle/_build/libmxoracle.so);
`RefBackend` wraps the reference's own sources compiled against the shims
(oracle/_ref/libmxref.so, only where the reference tree is available).
"""
from .runner import (OracleBackend, RefBackend, build_oracle, build_ref, ref_available, ORACLE_DIR)

__all__ = ["OracleBackend", "RefBackend", "build_oracle", "build_ref", "ref_available", "ORACLE_DIR"]

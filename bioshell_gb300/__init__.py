"""GB300-native all-vs-all crmsd engine for the bioshell-pdb crmsd path.

The compute runs in ``lib/libbioshell_crmsd.so`` (hand-written sm_103a CUDA
behind the C ABI of ``include/bioshell_crmsd.h``); this package is the thin
host-side mirror of the Rust API and the synthetic-workload generator.
"""
from .crmsd import (CrmsdMatrix, CrmsdOptions, Engine, crmsd, crmsd_all_vs_all, crmsd_batched,  # noqa: F401
                    default_engine, superpose, tri_index)
from .lib import CrmsdError  # noqa: F401
from .serving import CrmsdServer  # noqa: F401
from .superpose import Rototranslation  # noqa: F401

__all__ = ["CrmsdMatrix", "CrmsdOptions", "Engine", "crmsd", "crmsd_all_vs_all", "crmsd_batched", "default_engine", "tri_index",
           "CrmsdError", "CrmsdServer", "Rototranslation", "superpose"]

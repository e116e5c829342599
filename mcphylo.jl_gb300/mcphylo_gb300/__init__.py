"""mcphylo_gb300 -- GB300-native likelihood and branch-length gradient for
MCPhylo's PhyloDist (logpdf / gradlogpdf / MultiplePhyloDist).

The numerical work runs in hand-written sm_103a CUDA kernels inside
libmcphylo_gpu.so (C ABI in include/mcphylo_gpu.h); this package is the host
side: trees, parsers, substitution models and the PhyloDist interface.
"""
from . import models, parse, simulate, tree
from ._lib import DimensionMismatch, MCPhyError, NoDeviceError
from .engine import Engine, schedule_info
from .models import (GTR, HKY, JC, Restriction, calculate_transition, discrete_gamma_rates,
                     freeK, setmatrix)
from .parse import ParseNexus, datafortree
from .phylodist import MultiplePhyloDist, PhyloDist, gradlogpdf, logpdf
from .tree import (Node, ParseNewick, get_branchlength_vector, get_leaves, newick, post_order,
                   set_branchlength_vector, to_parent)

__all__ = [
    "Engine", "schedule_info", "PhyloDist", "MultiplePhyloDist", "logpdf", "gradlogpdf",
    "Restriction", "JC", "GTR", "HKY", "freeK", "setmatrix", "calculate_transition",
    "discrete_gamma_rates", "ParseNexus", "datafortree", "Node", "ParseNewick", "post_order",
    "get_leaves", "get_branchlength_vector", "set_branchlength_vector", "to_parent", "newick",
    "DimensionMismatch", "MCPhyError", "NoDeviceError", "models", "parse", "simulate", "tree",
]

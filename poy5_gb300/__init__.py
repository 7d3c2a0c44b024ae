"""GB300-native direct-optimization pairwise alignment (POY's algn.c path).

The compute path is the CUDA library ``libpoyalgn.so`` built from
``poy5_gb300/csrc`` (see :mod:`poy5_gb300.build`); this package is its
host-side interface.
"""
from .align import (Align, BatchResult, Context, CostMatrix, DOSMedian, PackedPairs,
                    PoyAlgnError, count_gaps, deltaw_calc, distance_batch, dos_median,
                    encode, median_batch, pack_pairs)
from .newkk import NewkkAlign, newkk_distance_batch, newkk_median_batch
from .peak import int32_rates
from .serve import ReplayResult, Reply, Server, Trace, poisson_trace
from .three_d import Powell3DBatch, align_3_powell, powell_3d_batch, powell_costs
from .tree import DownpassResult, Store, UppassResult, downpass, tree_levels, uppass

__all__ = ["Align", "BatchResult", "Context", "CostMatrix", "DOSMedian", "PackedPairs",
           "PoyAlgnError", "count_gaps", "deltaw_calc", "dos_median", "encode",
           "median_batch", "pack_pairs", "distance_batch", "DownpassResult", "Store", "downpass", "UppassResult", "uppass",
           "tree_levels", "NewkkAlign", "newkk_median_batch", "newkk_distance_batch", "ReplayResult", "Reply", "Server", "Trace", "poisson_trace",
           "int32_rates", "Powell3DBatch", "align_3_powell", "powell_3d_batch", "powell_costs"]
__version__ = "0.1.0"

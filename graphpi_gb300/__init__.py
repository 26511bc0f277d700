"""GB300-native GraphPi pattern-matching engine.

The engine (schedule compiler, C ABI, sm_103a kernels) lives in
libgraphpi_gb300.so; this package loads it with ctypes and mirrors the
reference's Graph / Pattern / Schedule / DataLoader / MotifGenerator API.
"""
from .api import (BatchExec, DataLoader, DataType, Graph, MotifGenerator, Pattern, PatternType, Plan, Schedule,
                  batch_count, chung_lu, complete_graph, count_host, from_edges, motifs_3_to_5, relabel_by_degree,
                  rmat, schedule_candidates, schedule_from_order)
from .native import GpmError, get_option, last_launch_stats, lib, set_option

__all__ = [
    "BatchExec", "DataLoader", "DataType", "Graph", "MotifGenerator", "Pattern", "PatternType", "Plan", "Schedule",
    "batch_count", "chung_lu", "complete_graph", "count_host", "from_edges", "motifs_3_to_5",
    "relabel_by_degree", "rmat", "schedule_candidates", "schedule_from_order", "GpmError", "get_option", "last_launch_stats", "lib", "set_option",
]

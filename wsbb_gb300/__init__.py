"""wsbb_gb300 — GB300 (sm_103a) flowshop branch-and-bound hot path.

Batched LB2 / LB1 / makespan bounds of begin-end nodes and the exact DFS
search built on them, behind the C-ABI in include/wsbb_gb300.h. The Python
modules are thin ctypes front ends over wsbb_gb300/_build/libwsbb_gb300.so.
"""
from ._lib import LIB_PATH, WsbbError, lib  # noqa: F401
from .bound import (BoundFlowshopGB300, Context, expand_children, gen_instance,  # noqa: F401
                    gen_pool, neh, node_stride, pack_records, taillard_instance,
                    unpack_records)

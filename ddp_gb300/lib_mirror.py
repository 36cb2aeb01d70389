"""The reference's LIB classes, mirrored over the C-ABI.

Same class names, constructor arguments and return conventions as
lkoshale/DDP LIB/include:
  Graph<T>            graph.h:13-43, read_graph :93-118
  GPU_Graph<T>        graph.cuh:12-89 (uploads on construction)
  Dynamic_Graph<T>    dynamic_graph.h:7-29 (get_graph returns the graph)
  GPU_Dynamic_Graph<T> dynamic_graph.cuh:8-26
  A_Star<T,U>         a_star.h:13-51, get_path :192-275
  GPU_A_Star<T,U>     a_star.cuh:12-52, get_path a_star.cu:109-303
get_path() returns [-1] if set_huiristics was not called, [] if the target
is unreachable, else the node ids from start to end.

Both A_Star and GPU_A_Star run on the GPU through ddp_solve (the reference's
A_Star is its serial CPU search; here there is no CPU search in the product).
K is passed through as the number of nodes expanded per iteration.
"""
from __future__ import annotations

from typing import List, Optional

import numpy as np

from . import CSR, H_USER, INF, DeviceGraph, read_graph_text


class Graph:
    """Host CSR in the reference layout: N offsets (no sentinel), E edges,
    E weights."""

    def __init__(self):
        self.N = 0
        self.E = 0
        self.offsets = np.zeros(0, np.int32)
        self.edges = np.zeros(0, np.int32)
        self.weights = np.zeros(0, np.uint32)

    @classmethod
    def from_csr(cls, g: CSR) -> "Graph":
        x = cls()
        x.N, x.E = g.n, g.e
        x.offsets = np.ascontiguousarray(g.off[:g.n], np.int32)
        x.edges = np.ascontiguousarray(g.col, np.int32)
        x.weights = np.ascontiguousarray(g.w, np.uint32)
        return x

    def read_graph(self, filename: str) -> None:
        # the reference prints an error and exit(1)s (graph.h:96-99); here
        # the C-ABI returns DDP_ERR_IO and this raises
        g = read_graph_text(filename)
        self.N, self.E = g.n, g.e
        self.offsets, self.edges, self.weights = g.off[:g.n].copy(), g.col, g.w

    def get_num_nodes(self) -> int:
        return self.N

    def get_num_edges(self) -> int:
        return self.E

    def get_offsets(self) -> np.ndarray:
        return self.offsets

    def get_edges(self) -> np.ndarray:
        return self.edges

    def get_weights(self) -> np.ndarray:
        return self.weights

    def free(self) -> None:
        self.offsets = self.edges = self.weights = None

    def to_csr(self) -> CSR:
        off = np.concatenate([self.offsets, [self.E]]).astype(np.int32)
        return CSR(self.N, off, self.edges, self.weights)


class GPU_Graph(Graph):
    """Graph copied to the device on construction."""

    def __init__(self, graph_cpu: Optional[Graph] = None):
        super().__init__()
        self.device: Optional[DeviceGraph] = None
        if graph_cpu is not None:
            self.N, self.E = graph_cpu.N, graph_cpu.E
            self.offsets, self.edges, self.weights = graph_cpu.offsets, graph_cpu.edges, graph_cpu.weights
            self.device = DeviceGraph.from_csr(graph_cpu.to_csr())

    def get_weight(self) -> np.ndarray:  # singular, as graph.cuh:32
        return self.weights


class Dynamic_Graph:
    def __init__(self, graph: Optional[Graph] = None, diff=None):
        self.graph = graph if graph is not None else Graph()
        self.diff = diff

    def get_graph(self) -> Graph:
        return self.graph

    def get_diff_graph(self):
        return self.diff


class GPU_Dynamic_Graph(Dynamic_Graph):
    def __init__(self, graph: Optional[GPU_Graph] = None, diff=None):
        super().__init__(graph if graph is not None else GPU_Graph(), diff)


class _AStarBase:
    def __init__(self, graph: Dynamic_Graph, start: int, end: int, K: int):
        self.graph = graph
        self.start_node = int(start)
        self.end_node = int(end)
        self.num_pq = int(K)
        self.Hx: Optional[np.ndarray] = None
        self.is_set_hx = False
        self.cost: int = INF

    def set_huiristics(self, hx) -> None:
        self.Hx = np.ascontiguousarray(hx, dtype=np.int32)
        self.is_set_hx = True

    def _device(self) -> DeviceGraph:
        g = self.graph.get_graph()
        if isinstance(g, GPU_Graph) and g.device is not None:
            return g.device
        if getattr(self, "_dg", None) is None:
            self._dg = DeviceGraph.from_csr(g.to_csr())
        return self._dg

    def get_path(self) -> List[int]:
        if not self.is_set_hx:
            return [-1]
        dg = self._device()
        h = dg.heuristic(self.end_node, H_USER, user_h=self.Hx)
        try:
            r = dg.solve(self.start_node, self.end_node, h, K=self.num_pq)
        finally:
            h.close()
        self.cost = r.cost
        if r.cost == INF:
            return []
        return [int(x) for x in r.path]


class A_Star(_AStarBase):
    pass


class GPU_A_Star(_AStarBase):
    pass

"""graphreduce_gb300: a Gather-Apply-Scatter graph engine for one GB300 GPU.

The compute path is libgas (hand-written CUDA for sm_103a behind the C ABI of
include/gas.h); this package is its Python host layer:

* :mod:`graphreduce_gb300.engine` -- ``GASEngineGPU`` with the reference's
  step API for BFS, SSSP, CC and PageRank, plus device-resident runs;
* :mod:`graphreduce_gb300.graph` -- edge lists, R-MAT / Erdos-Renyi / grid
  island generators and ``.gr`` I/O;
* :mod:`graphreduce_gb300.batch` -- many graphs x many BFS sources and
  personalized-PageRank seeds in one CUDA-graph launch;
* :mod:`graphreduce_gb300.learn` -- the learned schedule head and PageRank
  warm start (training and evaluation);
* :mod:`graphreduce_gb300.build` -- the in-tree nvcc build.

C++ users include ``include/gpugas.h`` instead (drop-in for the reference's
``gpugas.h``) and link libgas.
"""
from ._lib import GasError, load  # noqa: F401
from .batch import Batch  # noqa: F401
from .engine import GASEngineGPU, run_program  # noqa: F401
from .graph import EdgeList, edge_list_to_csr  # noqa: F401

__version__ = "0.1.0"

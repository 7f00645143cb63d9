"""GB300-native per-cell stiff chemistry integration (C++/CUDA host + sm_103a kernels).

The public surface is the C ABI of ``lib/libfcs_cuda.so`` (``include/fcs.h``);
this package holds its ctypes binding (:mod:`fcs._lib`), the in-tree build
(:mod:`fcs.build`) and the seeded synthetic workloads (:mod:`fcs.mechanism`,
:mod:`fcs.workloads`).
"""
from .mechanism import Mechanism, flatten, synthetic_mechanism  # noqa: F401
from .workloads import WORKLOADS, Cells, Workload, cells_for  # noqa: F401

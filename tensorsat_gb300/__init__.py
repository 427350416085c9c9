"""tensorsat_gb300: a GB300 (sm_103a) executor for TensorSat's contraction hot path.

The package mirrors the parts of the ``tensorsat`` API that the CNF contraction path uses
(``lib.sat.CNFInstance``, diagrams and wirings, the ``contractions`` entry points and the
autoray backend functions) and runs every contraction in hand-written CUDA kernels behind
the C ABI of ``include/tensorsat_gb300.h``:

>>> from tensorsat_gb300.lib.sat import CNFInstance
>>> from tensorsat_gb300.lang.cuda_rel import CudaRel
>>> from tensorsat_gb300.contractions.gpu import GpuContraction
>>> cnf = CNFInstance.random(3, 20, 85, rng=0)
>>> diagram = (cnf.inputs(None) >> cnf.diagram()).flatten()
>>> contraction = GpuContraction(CudaRel, diagram.wiring)
>>> bool(contraction.contract(diagram)), contraction.count(diagram)  # doctest: +SKIP
"""

__version__ = "0.1.0"

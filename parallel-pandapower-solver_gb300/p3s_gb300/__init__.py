"""GB300-native batched polar Newton-Raphson AC power flow.

A drop-in for the batched Newton path of e2nIEE/parallel-pandapower-solver (p3s): the
``nr_klu`` module surface (``p3s_gb300.nr_klu``), ``PolarNewtonSolverCUDA``
(``p3s_gb300.cuda.nr_polar_solver``) and the N-1 contingency driver
(``p3s_gb300.contingency``), all running on hand-written sm_103a kernels through the C ABI
of include/gbpf.h (``libgbpf.so``).
"""

__version__ = "0.1.0"

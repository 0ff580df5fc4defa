"""GB300-native (sm_103a) implementation of the QMCTorch VMC hot path.

Drop-in modules with the reference API: ``qmctorch_gb300.scf.Molecule``,
``qmctorch_gb300.wavefunction.SlaterJastrow``,
``qmctorch_gb300.sampler.Metropolis``, ``qmctorch_gb300.solver.Solver``.
Every evaluation runs hand-written CUDA kernels through the C ABI declared in
``include/qmc_gb300.h`` (library ``qmctorch_gb300/lib/libqmc_gb300.so``).
"""
__version__ = "0.1.0"

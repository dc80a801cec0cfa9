"""GB300 (sm_103a) rebuild of the diffSPH v2 per-timestep particle path.

Submodules:
- ``_lib``: ctypes binding of the C ABI (include/sph103.h, libsph103.so); raises when the
  library is missing;
- ``neighborhood``: ``neighborSearch`` with the reference's signature and return dict;
- ``solver``: ``Solver`` and ``BatchSolver``, the fused time step on a caller workspace;
- ``scheme``: ``simulationStep``, ``integrate``, ``solveShifting`` and
  ``computePressureAccelSwitch`` drop-ins;
- ``regions``: the open-boundary drop-ins (``LiuLiuConsistent``, ghosts, outlet, forcing,
  inlet);
- ``dropin``: installs the drop-ins into an imported reference package;
- ``adjoint``: the hand-written adjoint rollout behind ``torch.autograd``;
- ``learned``: the continuous-convolution learned step, its training and the judged rollout;
- ``scenes``: workload generators; ``build``: the in-tree nvcc build.
"""

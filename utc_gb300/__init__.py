"""GB300-native (sm_103a) N-body all-pairs step behind UTC's nbody task interface.

Layout:
  csrc/       CUDA kernels and the C ABI (include/nbody_gb300.h)
  task/       C++ drop-in task BodySystemGB300<T>, the UTC Task stand-in,
              initialisers and the app driver
  build.py    in-tree nvcc/g++ build (sm_103a only)
  _native.py  ctypes binding of the C ABI
  nbody.py    NBodySystem, the Python face of one context
  ics.py      seeded synthetic initial conditions
"""


def build_all(force: bool = False) -> None:
    """Compile the CUDA library, the task library and the app driver in-tree."""
    from .build import build

    build(force=force)

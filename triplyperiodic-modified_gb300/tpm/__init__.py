"""Host-side Python mirror of the GB300 RK4-substep library (libtpm.so).

``tpm.params``  - run parameters (ctypes mirror of tpm_params) and the
                  reference's parameter deck;
``tpm.inputs``  - seeded synthetic initial states and restart-file formats;
``tpm.capi``    - ctypes binding of the C ABI in include/tpm.h and a ``Grid``
                  facade with the reference grid's method names.
"""
from . import params, inputs  # noqa: F401

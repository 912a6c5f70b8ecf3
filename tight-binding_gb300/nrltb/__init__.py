"""nrltb -- host-side Python view of the GB300 NRL tight-binding k-point path.

The compute lives in ``_lib/libnrltb_gb300.so`` (CUDA, sm_103a) behind the C ABI
declared in ``include/nrltb.h``; this package marshals numpy arrays into it,
builds it (``nrltb.build``) and generates the seeded synthetic workloads
(``nrltb.synth``).
"""
from . import abi  # noqa: F401
from .api import (Context, KMesh, NrltbError, Opts, Params, Result, SkinFile,  # noqa: F401
                  Structure, read_skin, write_qlmt)

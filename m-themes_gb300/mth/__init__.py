"""Python-side mirror of the reference's solve interface over libmth.so.

The reference drives one RVE through `SetupJob()`, `Evolution()` and
`DestroyJob()` (src/evp.c:23-26).  `Solver` maps that lifecycle onto the C-ABI
of include/mth.h: construction = mth_create + mth_upload_microstructure,
`step()` = one mechanical step of Evolution, `close()` = mth_destroy.
`Batch` advances many independent RVEs together (mth_batch_*).
"""
from .capi import MTH_FP64, MTH_MIXED, MthError, load, params_from_config  # noqa: F401
from .solver import Batch, Solver, local_solve  # noqa: F401

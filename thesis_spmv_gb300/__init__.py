"""GB300-native (sm_103a) SpMV and power-method library.

A from-scratch GPU implementation of the hot path of KobeBergmans/Thesis_SPMV
(merge-path CRS SpMV, CSB and CO-H variants, the power method) behind the
reference's pwm::SparseMatrix interface.  The compute lives in
libpwmgpu.so (C ABI: include/pwmgpu.h); this package is its Python front end.
"""
from ._lib import (LOWFMT_AUTO, LOWFMT_MERGE, POWER_AUTO, POWER_FUSED, POWER_MULTI, PREC_F32, PREC_F64, PREC_MIXED,  # noqa: F401
                   PwmGpuError, check, lib, lib_path)
from .matrix import (AutoCuda, COHCuda, CRSCuda, CSBCuda, CudaSparseMatrix, Triplet, class_key, selectType,  # noqa: F401
                     tuner_entries, tuner_record, tuner_reset, tuner_size)

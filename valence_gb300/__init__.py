"""GB300 (sm_103a) implementation of VALENCE's VSVB energy hot path.

The compute lives in libvsvb_gb300.so (C ABI, include/vsvb_gpu.h); this
package is the thin Python host mirroring the reference's API
(valence_api.F90: initialize / calculate_energy / finalize), a
torch.autograd.Function for the weight gradient and the optimiser
(minimize_energy with first_order_opt / spin_opt / demgs_opt).
"""
from .api import (VSVBError, System, Batch, Optimizer, Options, FP64, MIXED, MIXED_DF64, rsg, valence_api_initialize,
                  valence_api_calculate_energy, valence_api_finalize, VSVBEnergy, library_path)

__all__ = ["VSVBError", "System", "Batch", "Optimizer", "Options", "FP64", "MIXED", "MIXED_DF64", "rsg",
           "valence_api_initialize", "valence_api_calculate_energy", "valence_api_finalize", "VSVBEnergy",
           "library_path"]

"""GB300 (sm_103a) backend for Paraiso's Orthotope Machine kernels.

The compute path is libom_gb300.so (CUDA, built in-tree by
paraiso_gb300.build); this package is its host-side mirror of the
generated OM classes."""
from .om import (CYCLIC, OPEN, Config, Ensemble, Hydro, HydroTape, Life,  # noqa: F401
                 OMError, OrthotopeMachine, autotune, autotune_ensemble, default_config,
                 ensemble_sizes, load_library, EXPORTS)

__all__ = ["Life", "Hydro", "HydroTape", "Ensemble", "ensemble_sizes", "autotune", "autotune_ensemble", "OrthotopeMachine", "Config", "OMError", "default_config",
           "load_library", "CYCLIC", "OPEN", "EXPORTS"]

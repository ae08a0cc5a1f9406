"""GB300 (sm_103a) backend for Paraiso's Orthotope Machine kernels.

The compute path is libom_gb300.so (CUDA, built in-tree by
paraiso_gb300.build); this package is its host-side mirror of the
generated OM classes."""
from .om import (CYCLIC, OPEN, Config, Ensemble, GraphMachine, Hydro, HydroTape,  # noqa: F401
                 Life, OMError, OrthotopeMachine, autotune, autotune_ensemble, default_config,
                 ensemble_rate, ensemble_sizes, load_library, measure_rate, EXPORTS)
from . import omgraph  # noqa: F401,E402

__all__ = ["Life", "Hydro", "HydroTape", "Ensemble", "GraphMachine", "omgraph", "ensemble_sizes", "autotune", "autotune_ensemble", "measure_rate", "ensemble_rate", "OrthotopeMachine", "Config", "OMError", "default_config",
           "load_library", "CYCLIC", "OPEN", "EXPORTS"]

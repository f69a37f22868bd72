"""GB300-native particle-history engine for minimc problems.

The CUDA library (``_lib/libminimc_gb300.so``) is built in-tree by
``minimc_gb300._build.build()``; ``minimc_gb300.engine`` binds its C ABI.
"""
from .engine import (  # noqa: F401
    Batch, Context, Driver, World, MCError, RunOpts, SITE_DTYPE, EVENTS,
    RNG_PHILOX, RNG_MINSTD, SCHEDULE_AUTO, SCHEDULE_HISTORY, SCHEDULE_EVENT, TSL_POD, TSL_MLP, TSL_GUIDED, TSL_PHILOX, TSL_FAST,
    GEOMETRY_ROBUST, GEOMETRY_REFERENCE, MLP_PARAMS, TrainDesc, TrainOut, THERMAL_POD, THERMAL_SURROGATE,
    THERMAL_GUIDED, THERMAL_POD_QUEUE,
    BANK_AUTO, BANK_SLOTS, BANK_DIRECT,
    load_library, library_path, exported_symbols,
)

__all__ = [
    "Batch", "Context", "Driver", "World", "MCError", "RunOpts", "SITE_DTYPE", "EVENTS",
    "RNG_PHILOX", "RNG_MINSTD", "SCHEDULE_AUTO", "SCHEDULE_HISTORY", "SCHEDULE_EVENT",
    "TSL_POD", "TSL_MLP", "TSL_GUIDED", "TSL_PHILOX", "TSL_FAST", "GEOMETRY_ROBUST", "GEOMETRY_REFERENCE", "MLP_PARAMS", "TrainDesc", "TrainOut",
    "THERMAL_POD", "THERMAL_SURROGATE", "THERMAL_GUIDED", "THERMAL_POD_QUEUE", "BANK_AUTO", "BANK_SLOTS", "BANK_DIRECT", "load_library", "library_path", "exported_symbols",
]

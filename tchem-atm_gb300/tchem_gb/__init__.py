"""GB300 engine for TChem-atm's batched box-model TR-BDF2 time advance.

Front end: NCAR-format YAML mechanisms and scenarios (KineticModel, set_scenario_conditions).
Compute: hand-written sm_103a CUDA kernels behind the C ABI in include/tchem_gb.h
(AtmosphericChemistry.runDeviceBatch / runHostBatch, kforward, reaction_rates, jacobian).
"""
from .mechanism import KineticModel, scenario_batch_size, set_scenario_conditions  # noqa: F401
from .atmospheric_chemistry import (  # noqa: F401
    AtmosphericChemistry, jacobian, kforward, reaction_rates, tadv_to_device, time_advance_array)

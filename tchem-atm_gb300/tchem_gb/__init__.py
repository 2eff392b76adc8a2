"""GB300 engine for TChem-atm's batched box-model TR-BDF2 time advance.

Front end: NCAR-format YAML mechanisms and scenarios (KineticModel, set_scenario_conditions,
set_scenario_photolysis_rates, set_scenario_external_forcing).
Compute: hand-written sm_103a CUDA kernels behind the C ABI in include/tchem_gb.h
(AtmosphericChemistry.runDeviceBatch / runHostBatch, kforward, reaction_rates, jacobian; the E3SM
gas chemistry in tchem_gb.e3sm: AtmosphericChemistryE3SM, ReactionRates, RateofProgress,
NetProductionRates; the gas-aerosol (SIMPOL.1) chemistry in tchem_gb.aerosol: AerosolModel,
AerosolChemistry, AerosolRHS).
"""
from .mechanism import (KineticModel, scenario_batch_size, set_scenario_conditions,  # noqa: F401
                        set_scenario_external_forcing, set_scenario_photolysis_rates)
from .atmospheric_chemistry import (  # noqa: F401
    AtmosphericChemistry, jacobian, kernel_launches, kforward, reaction_rates, tadv_to_device,
    time_advance_array)

/* Host-model driver interface: the extern "C" functions a host model (PartMC) binds to drive the
 * gas-aerosol chemistry one time step at a time, with the reference's names, argument order and
 * conventions (src/core/TChem_Driver.hpp:106-132, src/core/TChem_Driver.cpp:88-640), exported by
 * libtchem_gb_driver.so (which links libtchem_gb.so).
 *
 * One driver per process. initialize() reads the gas mechanism, the aerosol model and the solver
 * settings (tchem_gb_numerics_read) and creates nBatch zero state rows [rho, p, T, gas species,
 * particles] of TChem_getLengthOfStateVector() values and nBatch zero number-concentration rows of
 * TChem_getNumberConcentrationVectorSize() values. TChem_doTimestep(del_t) advances every row over
 * [0, del_t] with the engine's gas-aerosol TR-BDF2 kernel on the current CUDA device (the reference
 * integrates with CVODE BDF on the host-side state, src/core/TChem_Driver.cpp:437-640):
 * tolerances atol_time / rtol_time for the step error and atol_newton / rtol_newton for Newton,
 * first step dtmin, largest step del_t, up to max_num_time_iterations steps per kernel call and
 * calls until every row reaches del_t (at most max_num_time_iterations calls). Every row is
 * written back (the reference writes back row 0 only); a row whose advance fails keeps its state
 * and a warning is printed. A failed initialize() prints the reason and leaves the driver
 * uninitialized (the getters then return -1); tchem_gb_last_error() holds the message.
 */
#ifndef TCHEM_GB_DRIVER_H
#define TCHEM_GB_DRIVER_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

void initialize(const char* gasFile, const char* aeroFile, const char* numericsFile, const int nBatch);
void finalize(void);

int TChem_getNumberOfSpecies(void);
int TChem_getLengthOfStateVector(void);
/* nBatch * TChem_getLengthOfStateVector() (declared but not defined by the reference). */
int TChem_getStateVectorSize(void);
void TChem_getStateVector(double* array, const int iBatch);
void TChem_setStateVector(double* array, const int iBatch);
/* All nBatch state rows, row-major (declared but not defined by the reference). */
void TChem_getAllStateVectorHost(double* view);
/* Writes the name of gas species *index (at most buffer_size - 1 characters and a terminating
 * NUL) and returns the name's length. */
int TChem_getSpeciesName(int* index, char* result, const size_t buffer_size);

int TChem_getNumberConcentrationVectorSize(void);
void TChem_setNumberConcentrationVector(double* array, const int iBatch);
int TChem_getNumberOfAeroSpecies(void);
int TChem_getAerosolSpeciesName(int* index, char* result, const size_t buffer_size);
double TChem_getAerosolSpeciesDensity(int* index);
double TChem_getAerosolSpeciesMW(int* index);
double TChem_getAerosolSpeciesKappa(int* index);

#ifdef __cplusplus
/* The reference takes del_t by C++ reference (the same ABI as a pointer). */
void TChem_doTimestep(const double& del_t);
#else
void TChem_doTimestep(const double* del_t);
#endif

#ifdef __cplusplus
}
#endif

#endif /* TCHEM_GB_DRIVER_H */

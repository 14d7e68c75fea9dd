/*
 * Stand-in for the reference's InputOutput.cuh (not shipped;
 * NFFT/NFFT2_2D.cu:9).  NFFT2_2D.cu uses nothing from it.
 * TEST INFRASTRUCTURE ONLY.
 */
#ifndef ORACLE_REF_SHIM_INPUTOUTPUT_CUH
#define ORACLE_REF_SHIM_INPUTOUTPUT_CUH
#endif

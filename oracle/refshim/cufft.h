/* cuFFT subset used by calcIR.cu (calcIR.cu:790-826): a C2R transform with cuFFT's
 * convention, evaluated directly in double precision.  Test infrastructure only. */
#ifndef REFSHIM_CUFFT_H
#define REFSHIM_CUFFT_H
#include "shim_types.h"
typedef int cufftHandle;
typedef int cufftType;
typedef float cufftReal;
typedef refshim_cfloat cufftComplex;
#define CUFFT_C2R 0x2c
int cufftPlan1d(cufftHandle *plan, int nx, cufftType type, int batch);
int cufftExecC2R(cufftHandle plan, cufftComplex *idata, cufftReal *odata);
int cufftDestroy(cufftHandle plan);
#endif

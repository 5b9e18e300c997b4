/* libxdrfile subset used by calcIR.cu, reading CIRTRJ01 raw trajectories instead of
 * compressed .xtc files (see calcir_gb300/csrc/host_traj.cpp for the layout).
 * Test infrastructure only. */
#ifndef REFSHIM_XDRFILE_H
#define REFSHIM_XDRFILE_H
#include "shim_types.h"
#define XDR_DIM 3
typedef float rvec[XDR_DIM];
typedef float matrix[XDR_DIM][XDR_DIM];
typedef struct refshim_xdrfile XDRFILE;
enum { exdrOK = 0, exdrHEADER, exdrSTRING, exdrDOUBLE, exdrINT, exdrFLOAT, exdrUINT, exdr3DX, exdrCLOSE,
       exdrMAGIC, exdrNOMEM, exdrENDOFFILE, exdrFILENOTFOUND, exdrNR };
XDRFILE *xdrfile_open(const char *path, const char *mode);
int xdrfile_close(XDRFILE *xfp);
#endif

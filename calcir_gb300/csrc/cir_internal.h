// Internal helpers shared by the host (.cpp) and device (.cu) translation units.
#ifndef CIR_INTERNAL_H_
#define CIR_INTERNAL_H_

#include "calcir.h"
#include <stdarg.h>

// Physical constants exactly as the reference defines them (calcIR.h:36-37,
// calcIR.cu:1035-1036, 1197-1198).
#define CIR_HBAR        5.308837367      // cm^-1 * ps
#define CIR_PI          3.14159265359
#define CIR_BOHR_NM     18.8973f         // bohr per nm
#define CIR_CM_HARTREE  2.1947463E5f     // cm^-1 per hartree
#define CIR_CUTOFF      0.7831f          // nm, O(m) .. H(n) cutoff of the field sum
#define CIR_TDM_OFFSET  0.067f           // nm, transition dipole position along OH
#define CIR_OM_TIP4P    0.0150f          // nm, M-site distance used with imodel 1
#define CIR_QH          0.52f            // e, H charge of the field (all models)
#define CIR_QM          1.04f            // e, magnitude of the M charge

#ifdef __cplusplus
extern "C" {
#endif
// Record an error message for cir_last_error() and return `code`.
int cir_fail(int code, const char *fmt, ...);
#ifdef __cplusplus
}
#endif

// Spectroscopic map coefficients (calcIR.cu:1207-1242).
struct CirMaps {
    float w[3], x[2], p[2], mup[3], wi[3];
};
// Fills m for imap 0/1 and ispecies 0..3; returns false for any other imap.
bool cir_maps(int imap, int ispecies, CirMaps *m);


// .xtc trajectories (host_xtc.cpp), reached through cir_traj_info / cir_traj_read
bool cir_is_xtc(const char *path);
int cir_xtc_info(const char *path, int *natoms, int *nframes, float *frame_dt);
int cir_xtc_read(const char *path, int first, int count, float *xyz, float *boxes, float *times);

#endif

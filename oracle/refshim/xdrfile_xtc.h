/* see xdrfile.h */
#ifndef REFSHIM_XDRFILE_XTC_H
#define REFSHIM_XDRFILE_XTC_H
#include "xdrfile.h"
int read_xtc_natoms(char *fn, int *natoms);
int read_xtc(XDRFILE *xd, int natoms, int *step, float *time, matrix box, rvec *x, float *prec);
#endif

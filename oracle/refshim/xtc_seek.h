/* see xdrfile.h */
#ifndef REFSHIM_XTC_SEEK_H
#define REFSHIM_XTC_SEEK_H
#include "xdrfile.h"
int read_xtc_n_frames(char *fn, int *n_frames, int *est_nframes, int64_t **offsets);
int xdr_seek(XDRFILE *xd, int64_t pos, int whence);
#endif

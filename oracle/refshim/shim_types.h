/* Shared types of the host shims used to compile the reference calcIR.cu for the CPU.
 * Test infrastructure only (see oracle/build_ref.sh). */
#ifndef REFSHIM_TYPES_H
#define REFSHIM_TYPES_H
#include <stdint.h>
#include <stddef.h>
typedef struct { float x, y; } refshim_cfloat;
#endif

/* Types of SuperLU's slu_zdefs.h that tools/superlu.h and tools/dirac_solver.c
 * name.  The factorisation itself is provided by oracle/shim/slu_embed.c.
 * Oracle build only. */
#ifndef GADE_ORACLE_SLU_ZDEFS_H
#define GADE_ORACLE_SLU_ZDEFS_H
typedef int int_t;
typedef struct { double r, i; } doublecomplex;
typedef struct SuperMatrix SuperMatrix;
#endif

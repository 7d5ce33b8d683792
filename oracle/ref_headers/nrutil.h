/* Restated prototypes of the two Numerical-Recipes helpers the reference
 * solver calls (semsyn/src/nrutil.c:47 matrix, :155 free_dmatrix).  The
 * reference tree does not ship nrutil.h.  Oracle build infrastructure only. */
#ifndef SKS_ORACLE_REF_NRUTIL_H
#define SKS_ORACLE_REF_NRUTIL_H
float **matrix();
void free_dmatrix();
#endif

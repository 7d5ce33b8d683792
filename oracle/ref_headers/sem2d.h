/*
 * Restated declarations for building the reference solver sources
 * (semsyn/src/sem2d.c, sem2d_psvsh.c, sem2dMP.c, lagrange.c) as a CPU oracle.
 *
 * The reference tree includes "sem2d.h" but does not ship it.  Every type
 * below is written from how the reference sources use it:
 *   struct vector     - uvw[i].u[k], 3 displacement components per grid point
 *                       (sem2d_psvsh.c:1013-1025, 2116-2160)
 *   struct cmatrix    - meshs[i].c[i][j][k][l] and meshs[i].rho
 *                       (sem2d_psvsh.c:700-705, 1115-1118)
 *   struct cmatrix3d  - the 13 Voigt constants + rho filled in discret()
 *                       (sem2d_psvsh.c:655-660, 758-769)
 *   struct cmatrix2d  - argument of the unused Cijkl() (sem2d_psvsh.c:1489-1512)
 *   struct FIK        - FikM[..].F0/F1/F2[3] (sem2d_psvsh.c:1256-1259)
 *   struct Point2d    - element anchor points (sem2d_psvsh.c:866-873)
 *   struct Je4_one    - 2x2 Jacobian (lagrange.c:224-239)
 * This header is test infrastructure for the oracle build only.
 */
#ifndef SKS_ORACLE_REF_SEM2D_H
#define SKS_ORACLE_REF_SEM2D_H
struct vector    { float u[3]; };
struct cmatrix   { float c[3][3][3][3]; float rho; };
struct cmatrix3d { float c11, c12, c13, c16, c22, c23, c26, c33, c36,
                         c44, c45, c55, c66, rho; };
struct cmatrix2d { float c11, c13, c16, c33, c36, c44, c45, c55, c66, rho; };
struct FIK       { float F0[3], F1[3], F2[3]; };
struct Point2d   { float x, z; };
struct Je4_one   { float je[4]; };
#endif

/*
 * Stand-ins for the Fortran source-function routines uvw2sac.c calls only
 * with Conv_Source=1 (fa_, stime_, diff_, convt_ from semsyn/plot/source.f,
 * which needs a Fortran compiler this build does not have).  They end the
 * program instead of computing; the oracle runs uvw2sac with Conv_Source=0.
 * Test infrastructure for the oracle build only.
 */
#include <stdio.h>
#include <stdlib.h>

static void refuse(const char *name)
{
    fprintf(stderr, "uvw2sac oracle: %s (source.f, Conv_Source=1) is not built\n", name);
    exit(2);
}
void fa_(void) { refuse("fa"); }
void stime_(void) { refuse("stime"); }
void diff_(void) { refuse("diff"); }
void convt_(void) { refuse("convt"); }

/*
 * uvw2sac_gb300 — the reference's seismogram converter `uvw2sac par=run.par`
 * (semsyn/plot/uvw2sac.c) on this library: reads seis.u, seis.v and seis.w in
 * the working directory and writes, per receiver n, the SAC files n.ce, n.cn
 * and n.cz, log.txt and pm.xy, from the same par words.  Errors print a
 * message and exit with status 1.
 */
#include "sks.h"

#include <stdio.h>

int main(int argc, char **argv)
{
    const int rc = sks_uvw2sac(argc, (const char *const *)argv, NULL);
    if (rc) {
        fprintf(stderr, "uvw2sac_gb300: %s\n", sks_last_error());
        return 1;
    }
    return 0;
}

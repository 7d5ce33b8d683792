/*
 * Forced-in declaration for building semsyn/plot/uvw2sac.c as a CPU oracle
 * on a 64-bit host.  uvw2sac.c calls open_file() (defined in
 * semsyn/plot/readmodel.c:9, returning FILE *) without a declaration, so a
 * C89 compiler takes it to return int and cuts the 64-bit FILE pointer to 32
 * bits (the program then crashes reading the receiver file with get_rec=1).
 * Declaring it restores what the program did where int and pointers had the
 * same width.  Test infrastructure for the oracle build only.
 */
#include <stdio.h>
FILE *open_file();

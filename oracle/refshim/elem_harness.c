/* Harness that lets tests/golden/make_golden.py call the reference's own
 * element, geometry and skyline routines (truss.c, shell.c, misc.c, solve.c,
 * arc.c) on chosen inputs. It supplies the globals main.c normally defines
 * (main.c:323-328) and a setter for them; everything else is the reference's
 * unmodified code linked from its own objects. Test infrastructure only. */
#include <stdio.h>
#include <stdlib.h>

long NJ, NE_TR, NE_FR, NE_SH, NE_SBR, NE_FBR, NE_BR, NEQ, NBC, SNDOF, FNDOF, NTSTPS, ntstpsinpt;
double dt, ttot;
int ANAFLAG = 2, ALGFLAG = 3, OPTFLAG = 1, SLVFLAG = 0, FSIFLAG, FSIINCFLAG, brFSI_FLAG, shFSI_FLAG;
FILE *IFP[4], *OFP[8];
int CHKPT, RFLAG;

void href_set_sizes(long nj, long ne_tr, long ne_fr, long ne_sh, long neq, int anaflag,
                    int algflag)
{
    NJ = nj;
    NE_TR = ne_tr;
    NE_FR = ne_fr;
    NE_SH = ne_sh;
    NE_SBR = NE_FBR = NE_BR = 0;
    NEQ = neq;
    ANAFLAG = anaflag;
    ALGFLAG = algflag;
    SLVFLAG = 0;
    OPTFLAG = 1;
    for (int i = 0; i < 8; ++i) OFP[i] = stderr;
}

/* Point the reference's input stream (IFP[0]) at a file so that its own
 * property readers (prop_tr, prop_sh) can be called. */
int href_open_input(const char *path)
{
    if (IFP[0]) fclose(IFP[0]);
    IFP[0] = fopen(path, "r");
    return IFP[0] ? 0 : 1;
}

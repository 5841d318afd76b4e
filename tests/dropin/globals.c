/* Test infrastructure: the globals CU-BENs' main.c defines (main.c:323-328),
 * so that the drop-in library can be called from a test process. */
long NJ, NE_TR, NE_FR, NE_SH, NEQ, NTSTPS, NBC;
int ANAFLAG = 2, ALGFLAG = 3, SLVFLAG = 0;
double dt;

void cbg_set(long nj, long ne_tr, long ne_fr, long ne_sh, long neq, int anaflag, int algflag, double dt_)
{
    NJ = nj;
    NE_TR = ne_tr;
    NE_FR = ne_fr;
    NE_SH = ne_sh;
    NEQ = neq;
    NTSTPS = 0;
    NBC = 0;
    ANAFLAG = anaflag;
    ALGFLAG = algflag;
    SLVFLAG = 0;
    dt = dt_;
}

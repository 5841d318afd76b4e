/* Link-time wrapper (-Wl,--wrap=output) around the reference's output()
 * (misc.c:345-451). After the original text output it
 *   - appends every converged step (flag == 1) to a binary FP64 dump named by
 *     CUBEN_DUMP: int32 step, int32 iterations, double lambda, double d[NEQ];
 *   - prints a wall-clock timestamp per step to stderr when CUBEN_TIMES is set;
 *   - exits 0 after CAP_STEPS converged steps, since the MSAL loop
 *     (main.c:2647) has no step cap of its own.
 * Test infrastructure only: it never changes the reference's arithmetic. */
#include <stdio.h>
#include <stdlib.h>
#include <stdint.h>
#include <time.h>

extern long NEQ;
void __real_output(double *plpf, int *pitecnt, double *pd, double *pef, int flag);

static int n_steps = 0;
static FILE *dump_fp = NULL;
static struct timespec t_first;

void __wrap_output(double *plpf, int *pitecnt, double *pd, double *pef, int flag)
{
    __real_output(plpf, pitecnt, pd, pef, flag);
    if (flag != 1) return;
    struct timespec now;
    clock_gettime(CLOCK_MONOTONIC, &now);
    if (n_steps == 0) t_first = now;
    n_steps++;
    const char *dump = getenv("CUBEN_DUMP");
    if (dump && !dump_fp) dump_fp = fopen(dump, "wb");
    if (dump_fp) {
        int32_t hdr[2] = {n_steps, *pitecnt};
        fwrite(hdr, sizeof hdr, 1, dump_fp);
        fwrite(plpf, sizeof(double), 1, dump_fp);
        fwrite(pd, sizeof(double), (size_t)NEQ, dump_fp);
        fflush(dump_fp);
    }
    if (getenv("CUBEN_TIMES")) {
        double t = (double)(now.tv_sec - t_first.tv_sec) + 1e-9 * (double)(now.tv_nsec - t_first.tv_nsec);
        fprintf(stderr, "step %d lpf %.17g it %d t %.6f\n", n_steps, *plpf, *pitecnt, t);
    }
    const char *cap = getenv("CAP_STEPS");
    if (cap && n_steps >= atoi(cap)) {
        fflush(NULL);
        exit(0);
    }
}

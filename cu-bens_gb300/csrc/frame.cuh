// Frame member geometry shared by the frame kernels and the drop-in updatc:
// the triad and length of prop_fr (frame.c:130-160) and updatc
// (misc.c:108-147), with the member's fixed auxiliary point.
#pragma once

#include <cuda_runtime.h>

namespace cb {

__host__ __device__ __forceinline__ void cross_norm(const double *a, const double *b, double *c)
{
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
    double l = sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    c[0] /= l;
    c[1] /= l;
    c[2] /= l;
}

// rows x^, y^, z^ of c; x^ along the member, z^ = x^ x (aux - end 1)
// normalised, y^ = z^ x x^ normalised
__host__ __device__ __forceinline__ void frame_geometry(const double *pa, const double *pb, const double *aux,
                                               double *c, double *len)
{
    double el[3] = {pb[0] - pa[0], pb[1] - pa[1], pb[2] - pa[2]};
    double L = sqrt(el[0] * el[0] + el[1] * el[1] + el[2] * el[2]);
    double lx[3] = {el[0] / L, el[1] / L, el[2] / L};
    double tmp[3] = {aux[0] - pa[0], aux[1] - pa[1], aux[2] - pa[2]};
    double lz[3], ly[3];
    cross_norm(lx, tmp, lz);
    cross_norm(lz, lx, ly);
    for (int m = 0; m < 3; ++m) {
        c[m] = lx[m];
        c[3 + m] = ly[m];
        c[6 + m] = lz[m];
    }
    *len = L;
}

}  // namespace cb

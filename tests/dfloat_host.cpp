// Host build of the double-float arithmetic of the FP32 path's cost
// (sfmtory_gb300/csrc/dfloat.cuh), for its CPU test (test_dfloat.py):
// each entry returns the pair (hi, lo) of one operation.
#include "dfloat.cuh"

using sfmba::dfl;

extern "C" {
void h_df_from(double x, float *out) {
    const dfl r = sfmba::df_from(x);
    out[0] = r.hi;
    out[1] = r.lo;
}
void h_df_add(float ah, float al, float bh, float bl, float *out) {
    const dfl r = dfl{ah, al} + dfl{bh, bl};
    out[0] = r.hi;
    out[1] = r.lo;
}
void h_df_mul(float ah, float al, float bh, float bl, float *out) {
    const dfl r = dfl{ah, al} * dfl{bh, bl};
    out[0] = r.hi;
    out[1] = r.lo;
}
void h_df_recip(float ah, float al, float *out) {
    const dfl r = sfmba::df_recip(dfl{ah, al});
    out[0] = r.hi;
    out[1] = r.lo;
}
}

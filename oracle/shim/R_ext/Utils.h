#ifndef NNGP_SHIM_UTILS_H
#define NNGP_SHIM_UTILS_H
#ifdef __cplusplus
extern "C" {
#endif
void rsort_with_index(double *x, int *indx, int n);
void R_CheckUserInterrupt(void);
#ifdef __cplusplus
}
#endif
#endif

/* Minimal stand-in for R's <R_ext/Rdynload.h> (test infrastructure): routine registration.
 * R_registerRoutines keeps the .Call table so a test can look routines up by name and arity. */
#ifndef NNGP_SHIM_RDYNLOAD_H
#define NNGP_SHIM_RDYNLOAD_H
#include "Boolean.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef void *(*DL_FUNC)(void);
typedef struct {
  const char *name;
  DL_FUNC fun;
  int numArgs;
} R_CallMethodDef;
typedef struct shim_dll_info DllInfo;
int R_registerRoutines(DllInfo *info, const void *croutines, const R_CallMethodDef *callRoutines,
                       const void *fortranRoutines, const void *externalRoutines);
int R_useDynamicSymbols(DllInfo *info, Rboolean value);
/* The table passed to the last R_registerRoutines call (NULL before one). */
const R_CallMethodDef *shim_call_routines(void);
#ifdef __cplusplus
}
#endif
#endif

/* Minimal stand-in for R's <R_ext/Boolean.h> (test infrastructure). */
#ifndef NNGP_SHIM_BOOLEAN_H
#define NNGP_SHIM_BOOLEAN_H
typedef enum { FALSE = 0, TRUE } Rboolean;
#endif

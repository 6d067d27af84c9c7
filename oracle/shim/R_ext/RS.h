#ifndef NNGP_SHIM_RS_H
#define NNGP_SHIM_RS_H
#define F77_NAME(x) x ## _
#define F77_CALL(x) x ## _
#endif

/* Minimal stand-in for R_ext/Rdynload.h (ORACLE build only). */
#ifndef RSTUB_RDYNLOAD_H
#define RSTUB_RDYNLOAD_H
#include "../Rinternals.h"
typedef void *(*DL_FUNC)(void);
typedef struct {
    const char *name;
    DL_FUNC fun;
    int numArgs;
} R_CallMethodDef;
typedef struct rstub_dll DllInfo;
int R_registerRoutines(DllInfo *info, const void *c, const R_CallMethodDef *call,
                       const void *fortran, const void *external);
Rboolean R_useDynamicSymbols(DllInfo *info, Rboolean value);
Rboolean R_forceSymbols(DllInfo *info, Rboolean value);
#endif

/* Minimal stand-in for R_ext/Utils.h (ORACLE build only). */
#ifndef RSTUB_UTILS_H
#define RSTUB_UTILS_H
#include "../Rinternals.h"
#endif

/* Minimal stand-in for R.h (ORACLE build only); see Rinternals.h. */
#ifndef RSTUB_R_H
#define RSTUB_R_H
#include "Rinternals.h"
#endif

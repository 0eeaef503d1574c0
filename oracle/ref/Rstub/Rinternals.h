/*
 * Minimal stand-in for R's C API, enough to compile the package's
 * src/forceatlas2.c outside R (R is not installed here). ORACLE build only:
 * the functions are implemented in ../ref_harness.c. Only what that file
 * uses is declared.
 */
#ifndef RSTUB_RINTERNALS_H
#define RSTUB_RINTERNALS_H

#include <stddef.h>

typedef ptrdiff_t R_xlen_t;
typedef enum { FALSE = 0, TRUE = 1 } Rboolean;
typedef struct rstub_sexp *SEXP;

enum {
    NILSXP = 0,
    SYMSXP = 1,
    CHARSXP = 9,
    LGLSXP = 10,
    INTSXP = 13,
    REALSXP = 14,
    STRSXP = 16,
    VECSXP = 19
};

#define NA_INTEGER (-2147483647 - 1)

extern SEXP R_NamesSymbol;

SEXP Rf_allocVector(int type, R_xlen_t n);
SEXP Rf_duplicate(SEXP x);
SEXP Rf_install(const char *name);
SEXP Rf_mkChar(const char *s);
SEXP Rf_mkNamed(int type, const char **names);
SEXP Rf_ScalarLogical(int v);
SEXP Rf_setAttrib(SEXP x, SEXP name, SEXP value);
int Rf_asInteger(SEXP x);
Rboolean Rf_isInteger(SEXP x);
Rboolean Rf_isReal(SEXP x);
Rboolean Rf_isLogical(SEXP x);
Rboolean Rf_isString(SEXP x);
void Rf_error(const char *fmt, ...) __attribute__((noreturn));

int LENGTH(SEXP x);
R_xlen_t XLENGTH(SEXP x);
int *INTEGER(SEXP x);
int *LOGICAL(SEXP x);
double *REAL(SEXP x);
const char *R_CHAR(SEXP x);
SEXP STRING_ELT(SEXP x, R_xlen_t i);
void SET_STRING_ELT(SEXP x, R_xlen_t i, SEXP v);
SEXP SET_VECTOR_ELT(SEXP x, R_xlen_t i, SEXP v);
SEXP Rf_protect(SEXP x);
void Rf_unprotect(int n);

#define allocVector Rf_allocVector
#define duplicate Rf_duplicate
#define install Rf_install
#define mkChar Rf_mkChar
#define mkNamed Rf_mkNamed
#define ScalarLogical Rf_ScalarLogical
#define setAttrib Rf_setAttrib
#define asInteger Rf_asInteger
#define isInteger Rf_isInteger
#define isReal Rf_isReal
#define isLogical Rf_isLogical
#define isString Rf_isString
#define error Rf_error
#define CHAR R_CHAR
#define PROTECT Rf_protect
#define UNPROTECT Rf_unprotect

char *R_alloc(size_t n, int size);
void R_CheckUserInterrupt(void);
Rboolean R_ToplevelExec(void (*fun)(void *), void *data);

#endif

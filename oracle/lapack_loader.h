/*
 * Oracle-only LAPACK/BLAS access (test infrastructure, never part of the product).
 *
 * The reference links MKL (make.inc.example:16).  That library is not available here, so the
 * oracle resolves the same LAPACK routines at run time from an OpenBLAS build: by default the
 * one bundled with scipy (LP64, symbols prefixed "scipy_"), or any library named in the
 * environment variable PARAHT_ORACLE_LAPACK.  All routines use the Fortran calling convention,
 * including the hidden character-length arguments.
 */
#ifndef PARAHT_ORACLE_LAPACK_LOADER_H
#define PARAHT_ORACLE_LAPACK_LOADER_H
#include <stddef.h>

typedef int lint; /* LP64 LAPACK integer */
typedef size_t flen; /* gfortran hidden character length */

typedef struct {
  void (*dgeqr2)(const lint*, const lint*, double*, const lint*, double*, double*, lint*);
  void (*dgeqrf)(const lint*, const lint*, double*, const lint*, double*, double*, const lint*, lint*);
  void (*dgerqf)(const lint*, const lint*, double*, const lint*, double*, double*, const lint*, lint*);
  void (*dgerq2)(const lint*, const lint*, double*, const lint*, double*, double*, lint*);
  void (*dorgrq)(const lint*, const lint*, const lint*, double*, const lint*, const double*, double*, const lint*, lint*);
  void (*dorgr2)(const lint*, const lint*, const lint*, double*, const lint*, const double*, double*, lint*);
  void (*dgelq2)(const lint*, const lint*, double*, const lint*, double*, double*, lint*);
  void (*dlarfg)(const lint*, double*, double*, const lint*, double*);
  void (*dlarf)(const char*, const lint*, const lint*, const double*, const lint*, const double*, double*, const lint*, double*, flen);
  void (*dlarft)(const char*, const char*, const lint*, const lint*, const double*, const lint*, const double*, double*, const lint*, flen, flen);
  void (*dlarfb)(const char*, const char*, const char*, const char*, const lint*, const lint*, const lint*, const double*, const lint*,
                 const double*, const lint*, double*, const lint*, double*, const lint*, flen, flen, flen, flen);
  void (*dlacpy)(const char*, const lint*, const lint*, const double*, const lint*, double*, const lint*, flen);
  void (*dlaset)(const char*, const lint*, const lint*, const double*, const double*, double*, const lint*, flen);
  void (*dgemm)(const char*, const char*, const lint*, const lint*, const lint*, const double*, const double*, const lint*,
                const double*, const lint*, const double*, double*, const lint*, flen, flen);
  double (*dlange)(const char*, const lint*, const lint*, const double*, const lint*, double*, flen);
  void (*dgghd3)(const char*, const char*, const lint*, const lint*, const lint*, double*, const lint*, double*, const lint*,
                 double*, const lint*, double*, const lint*, double*, const lint*, lint*, flen, flen);
  void (*dhgeqz)(const char*, const char*, const char*, const lint*, const lint*, const lint*, double*, const lint*, double*,
                 const lint*, double*, double*, double*, double*, const lint*, double*, const lint*, double*, const lint*, lint*,
                 flen, flen, flen);
  void (*dlartg)(const double*, const double*, double*, double*, double*);
  void (*drot)(const lint*, double*, const lint*, double*, const lint*, const double*, const double*);
  void (*set_num_threads)(int);
} lapack_table;

/* Returns NULL (and fills err) when no usable library is found. */
const lapack_table* oracle_lapack(char* err, size_t errlen);

#endif

/*
 * Oracle-only LAPACK loader (test infrastructure).  See lapack_loader.h.
 */
#define _GNU_SOURCE
#include "lapack_loader.h"
#include <dlfcn.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#ifndef ORACLE_DEFAULT_LAPACK
#define ORACLE_DEFAULT_LAPACK ""
#endif

static lapack_table g_tab;
static int g_state = 0; /* 0 = not loaded, 1 = ok, -1 = failed */
static char g_err[512];
static pthread_mutex_t g_mu = PTHREAD_MUTEX_INITIALIZER;

static void* sym(void* h, const char* name) {
  static const char* pre[] = {"scipy_", "", NULL};
  char buf[128];
  for (int i = 0; pre[i]; ++i) {
    snprintf(buf, sizeof buf, "%s%s_", pre[i], name);
    void* f = dlsym(h, buf);
    if (f) return f;
  }
  return NULL;
}

static void* sym_threads(void* h) {
  static const char* names[] = {"scipy_openblas_set_num_threads", "openblas_set_num_threads", NULL};
  for (int i = 0; names[i]; ++i) {
    void* f = dlsym(h, names[i]);
    if (f) return f;
  }
  return NULL;
}

static int load(void) {
  const char* path = getenv("PARAHT_ORACLE_LAPACK");
  if (!path || !*path) path = ORACLE_DEFAULT_LAPACK;
  if (!path || !*path) {
    snprintf(g_err, sizeof g_err, "no LAPACK library configured (set PARAHT_ORACLE_LAPACK)");
    return -1;
  }
  void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!h) {
    snprintf(g_err, sizeof g_err, "dlopen(%s) failed: %s", path, dlerror());
    return -1;
  }
#define GET(field, name)                                                          \
  do {                                                                            \
    *(void**)(&g_tab.field) = sym(h, name);                                       \
    if (!g_tab.field) {                                                           \
      snprintf(g_err, sizeof g_err, "symbol %s missing in %s", name, path);       \
      return -1;                                                                  \
    }                                                                             \
  } while (0)
  GET(dgeqr2, "dgeqr2");
  GET(dgeqrf, "dgeqrf");
  GET(dgerqf, "dgerqf");
  GET(dgerq2, "dgerq2");
  GET(dorgrq, "dorgrq");
  GET(dorgr2, "dorgr2");
  GET(dgelq2, "dgelq2");
  GET(dlarfg, "dlarfg");
  GET(dlarf, "dlarf");
  GET(dlarft, "dlarft");
  GET(dlarfb, "dlarfb");
  GET(dlacpy, "dlacpy");
  GET(dlaset, "dlaset");
  GET(dgemm, "dgemm");
  GET(dlange, "dlange");
  GET(dgghd3, "dgghd3");
  GET(dhgeqz, "dhgeqz");
  GET(dlartg, "dlartg");
  GET(drot, "drot");
#undef GET
  *(void**)(&g_tab.set_num_threads) = sym_threads(h);
  return 1;
}

const lapack_table* oracle_lapack(char* err, size_t errlen) {
  pthread_mutex_lock(&g_mu);
  if (g_state == 0) g_state = load();
  pthread_mutex_unlock(&g_mu);
  if (g_state == 1) return &g_tab;
  if (err && errlen) snprintf(err, errlen, "%s", g_err);
  return NULL;
}

/*
 * paraht_oracle.c -- CPU oracle for the two-stage Hessenberg-triangular reduction.
 *
 * TEST INFRASTRUCTURE ONLY.  This file restates, call for call, the reference's
 *   src/ab2rht.f90:8-495       ab2rht_simple            (stage 1: (A,B) -> (r-Hessenberg, triangular))
 *   src/rht2ht.f90:1346-2051   rht2ht_householder       (stage 2: r-Hessenberg -> Hessenberg)
 *   src/rht2ht.f90:2053-2180   rht2ht_householder_unblocked (independent stage-2 cross-check)
 * with the same LAPACK calls and argument expressions, and the same OpenMP task graph
 * (priorities, depend tokens, taskloop row/column chunks).  Only the Fortran control flow
 * is re-expressed in C.  Indices below are 1-based, like the reference, through the IX macro.
 *
 * Only tests, the smoke check and the CPU-baseline leg of the benchmark may load this
 * library; the GPU product never calls it.
 *
 * Deliberate deviation (documented where it happens): wherever the reference passes a
 * reflector count K larger than the row/column count of the block (possible only in the last
 * block of a sweep group, where the extra reflectors all have tau = 0), the oracle passes
 * min(K, rows).  The product of the reflectors is identical, and the reference's form would
 * touch memory past the end of the matrix column.
 */
#include <math.h>
#include <omp.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "lapack_loader.h"

#define IX(M, ld, i, j) (M)[((size_t)(i)-1) + ((size_t)(j)-1) * (size_t)(ld)]
#define MIN(a, b) ((a) < (b) ? (a) : (b))
#define MAX(a, b) ((a) > (b) ? (a) : (b))

static const lapack_table* LP;

static double now_s(void) {
  struct timespec ts;
  clock_gettime(CLOCK_MONOTONIC, &ts);
  return ts.tv_sec + 1e-9 * ts.tv_nsec;
}

/* ---- thin call wrappers (Fortran ABI: everything by reference + hidden lengths) ---- */
static void geqr2(lint m, lint n, double* a, lint lda, double* tau, double* work) {
  lint info;
  LP->dgeqr2(&m, &n, a, &lda, tau, work, &info);
}
static void gerqf(lint m, lint n, double* a, lint lda, double* tau, double* work, lint lwork) {
  lint info;
  LP->dgerqf(&m, &n, a, &lda, tau, work, &lwork, &info);
}
static void gerq2(lint m, lint n, double* a, lint lda, double* tau, double* work) {
  lint info;
  LP->dgerq2(&m, &n, a, &lda, tau, work, &info);
}
static void orgrq(lint m, lint n, lint k, double* a, lint lda, const double* tau, double* work, lint lwork) {
  lint info;
  LP->dorgrq(&m, &n, &k, a, &lda, tau, work, &lwork, &info);
}
static void orgr2(lint m, lint n, lint k, double* a, lint lda, const double* tau, double* work) {
  lint info;
  LP->dorgr2(&m, &n, &k, a, &lda, tau, work, &info);
}
static void gelq2(lint m, lint n, double* a, lint lda, double* tau, double* work) {
  lint info;
  LP->dgelq2(&m, &n, a, &lda, tau, work, &info);
}
static void larfg(lint n, double* alpha, double* x, lint incx, double* tau) { LP->dlarfg(&n, alpha, x, &incx, tau); }
static void larf(const char* side, lint m, lint n, const double* v, lint incv, const double* tau, double* c, lint ldc,
                 double* work) {
  if (m <= 0 || n <= 0) return;
  LP->dlarf(side, &m, &n, v, &incv, tau, c, &ldc, work, 1);
}
static void larft(const char* direct, const char* storev, lint n, lint k, const double* v, lint ldv, const double* tau,
                  double* t, lint ldt) {
  LP->dlarft(direct, storev, &n, &k, v, &ldv, tau, t, &ldt, 1, 1);
}
static void larfb(const char* side, const char* trans, const char* direct, const char* storev, lint m, lint n, lint k,
                  const double* v, lint ldv, const double* t, lint ldt, double* c, lint ldc, double* work, lint ldwork) {
  if (m <= 0 || n <= 0 || k <= 0) return;
  LP->dlarfb(side, trans, direct, storev, &m, &n, &k, v, &ldv, t, &ldt, c, &ldc, work, &ldwork, 1, 1, 1, 1);
}
static void lacpy(lint m, lint n, const double* a, lint lda, double* b, lint ldb) {
  LP->dlacpy("A", &m, &n, a, &lda, b, &ldb, 1);
}

static int init_lapack(void) {
  char err[512];
  LP = oracle_lapack(err, sizeof err);
  if (!LP) {
    fprintf(stderr, "paraht oracle: %s\n", err);
    return -1;
  }
  return 0;
}

const char* oracle_lapack_error(void) {
  static char err[512];
  if (oracle_lapack(err, sizeof err)) return "";
  return err;
}

/* Sets the BLAS thread count (tasks call BLAS single-threaded, like MKL inside OpenMP tasks). */
void oracle_set_blas_threads(int t) {
  if (init_lapack() == 0 && LP->set_num_threads) LP->set_num_threads(t);
}

/* ab2rht.f90:63-67 and rht2ht.f90:1377-1381: taskloop chunk size. */
static int chunk_size(int n) {
  int nthreads = omp_get_max_threads();
  int bs = n / nthreads;
  if (bs % 16 != 0) bs += 16 - bs % 16;
  bs = MAX(32, bs);
  bs = MIN(n, bs);
  return bs;
}

/* ======================================================================================
 * Stage 1: ab2rht_simple (src/ab2rht.f90:8-495)
 * phase[0..2] <- genleft, genright, multiplication times (time_components, ab2rht.f90:487-490)
 * ====================================================================================== */
int oracle_ab2rht_simple(int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z, int ldz, int nb,
                         int p, int time_components, double* phase) {
  if (init_lapack()) return -100;
  if (n < 1 || nb < 1 || p < 2) return -1;
  if (n - nb - 1 < 1) return 0; /* ab2rht.f90:71: the panel loop is empty */
  const int pnb = p * nb;
  int nblk0 = (n - nb) / ((p - 1) * nb);
  if ((n - nb) % ((p - 1) * nb) != 0) nblk0++; /* ab2rht.f90:34-35 */
  double* VL = calloc((size_t)pnb * nb * nblk0, sizeof(double));
  double* VR = calloc((size_t)nb * pnb * nblk0, sizeof(double));
  double* TL = calloc((size_t)nb * nb * nblk0, sizeof(double));
  double* TR = calloc((size_t)nb * nb * nblk0, sizeof(double));
  double* Bc = calloc((size_t)pnb * pnb, sizeof(double));
  /* ab2rht.f90:42-47: workspace size (query dgerqf / dorgrq) */
  lint lwork = (lint)pnb * n;
  {
    double q;
    lint m = pnb, minus1 = -1, info;
    LP->dgerqf(&m, &m, Bc, &m, &q, &q, &minus1, &info);
    lwork = MAX(lwork, (lint)q);
    LP->dorgrq(&m, &m, &m, Bc, &m, &q, &q, &minus1, &info);
    lwork = MAX(lwork, (lint)q);
  }
  double t_genleft = 0, t_genright = 0, t_mul = 0, t0 = 0;
  char tokA, tokB, tokB22, tokB33, tokQ, tokZ, tokVL, tokTL, tokVR, tokTR;
#define VLx(i, j, bl) VL[((size_t)(i)-1) + ((size_t)(j)-1) * pnb + ((size_t)(bl)-1) * pnb * nb]
#define VRx(i, j, bl) VR[((size_t)(i)-1) + ((size_t)(j)-1) * nb + ((size_t)(bl)-1) * nb * pnb]
#define TLx(i, j, bl) TL[((size_t)(i)-1) + ((size_t)(j)-1) * nb + ((size_t)(bl)-1) * nb * nb]
#define TRx(i, j, bl) TR[((size_t)(i)-1) + ((size_t)(j)-1) * nb + ((size_t)(bl)-1) * nb * nb]

#pragma omp parallel
#pragma omp single
  {
    const int blocksize = chunk_size(n);
    for (int jb = 1; jb <= n - nb - 1; jb += nb) {
      int nblocks = (n - nb - jb + 1) / ((p - 1) * nb); /* ab2rht.f90:74-75 */
      if ((n - nb - jb + 1) % ((p - 1) * nb) != 0) nblocks++;
      const int ibtop = jb + nb + (nblocks - 1) * (p - 1) * nb;
      const int stride = nb * (p - 1);
      if (time_components) {
#pragma omp taskwait
        t0 = now_s();
      }
      /* ---- left generation, ab2rht.f90:85-123 ---- */
#pragma omp task depend(inout : tokA) depend(out : tokVL) depend(out : tokTL) priority(100) firstprivate(jb, nblocks)
      {
        double work[2 * 1024];
        double* w = nb <= 1024 ? work : malloc(sizeof(double) * 2 * nb);
        int bl = 0;
        for (int ib = ibtop; ib >= jb + nb; ib -= stride) {
          bl++;
          int ib2 = MIN(n, ib + pnb - 1), nb2 = ib2 - ib + 1, k = MIN(nb, nb2);
          geqr2(nb2, nb, &IX(A, lda, ib, jb), lda, w, w + nb);     /* :105 */
          lacpy(nb2, nb, &IX(A, lda, ib, jb), lda, &VLx(1, 1, bl), pnb); /* :108 */
          for (int j = jb; j <= jb + nb - 1; j++)                   /* :109-113 */
            for (int i = ib + j - jb + 1; i <= ib2; i++) IX(A, lda, i, j) = 0.0;
          larft("F", "C", nb2, k, &VLx(1, 1, bl), pnb, w, &TLx(1, 1, bl), nb); /* :116 */
        }
        if (w != work) free(w);
      }
      if (time_components) {
#pragma omp taskwait
        double t1 = now_s();
        t_genleft += t1 - t0;
        t0 = t1;
      }
      /* ---- apply left reflectors to B, ab2rht.f90:135-171 ---- */
#pragma omp task depend(inout : tokB) depend(in : tokVL) depend(in : tokTL) priority(100) firstprivate(jb, nblocks)
      {
#pragma omp taskloop firstprivate(jb, nblocks)
        for (int i = 1; i <= n; i += blocksize) {
          double* work = malloc(sizeof(double) * (size_t)blocksize * nb);
          int c2 = MIN(i + blocksize - 1, n);
          int bl = 0;
          for (int ib = ibtop; ib >= jb + nb; ib -= stride) {
            bl++;
            int ib2 = MIN(n, ib + pnb - 1), nb2 = ib2 - ib + 1, k = MIN(nb, nb2);
            int c1 = MAX(ib, i);
            if (c2 >= c1)
              larfb("L", "T", "F", "C", nb2, c2 - c1 + 1, k, &VLx(1, 1, bl), pnb, &TLx(1, 1, bl), nb,
                    &IX(B, ldb, ib, c1), ldb, work, c2 - c1 + 1); /* :161 */
          }
          free(work);
        }
      }
      /* ---- apply left reflectors to A, ab2rht.f90:176-212 ---- */
#pragma omp task depend(inout : tokA) depend(in : tokVL) depend(in : tokTL) priority(1) firstprivate(jb, nblocks)
      {
#pragma omp taskloop firstprivate(jb, nblocks)
        for (int i = 1; i <= n; i += blocksize) {
          int c1 = MAX(i, jb + nb), c2 = MIN(i + blocksize - 1, n);
          if (c2 >= c1) {
            double* work = malloc(sizeof(double) * (size_t)blocksize * nb);
            int bl = 0;
            for (int ib = ibtop; ib >= jb + nb; ib -= stride) {
              bl++;
              int ib2 = MIN(n, ib + pnb - 1), nb2 = ib2 - ib + 1, k = MIN(nb, nb2);
              larfb("L", "T", "F", "C", nb2, c2 - c1 + 1, k, &VLx(1, 1, bl), pnb, &TLx(1, 1, bl), nb,
                    &IX(A, lda, ib, c1), lda, work, c2 - c1 + 1); /* :202 */
            }
            free(work);
          }
        }
      }
      /* ---- apply left reflectors to Q, ab2rht.f90:217-250 ---- */
#pragma omp task depend(inout : tokQ) depend(in : tokVL) depend(in : tokTL) priority(1) firstprivate(jb, nblocks)
      {
#pragma omp taskloop firstprivate(jb, nblocks)
        for (int i = 1; i <= n; i += blocksize) {
          int r1 = i, r2 = MIN(i + blocksize - 1, n);
          double* work = malloc(sizeof(double) * (size_t)blocksize * nb);
          int bl = 0;
          for (int ib = ibtop; ib >= jb + nb; ib -= stride) {
            bl++;
            int ib2 = MIN(n, ib + pnb - 1), nb2 = ib2 - ib + 1, k = MIN(nb, nb2);
            larfb("R", "N", "F", "C", r2 - r1 + 1, nb2, k, &VLx(1, 1, bl), pnb, &TLx(1, 1, bl), nb,
                  &IX(Q, ldq, r1, ib), ldq, work, r2 - r1 + 1); /* :241 */
          }
          free(work);
        }
      }
      if (time_components) {
#pragma omp taskwait
        double t1 = now_s();
        t_mul += t1 - t0;
        t0 = t1;
      }
      /* ---- right generation (+ B updates), ab2rht.f90:263-375 ---- */
#pragma omp task depend(inout : tokB) depend(out : tokVR) depend(out : tokTR) priority(100) firstprivate(jb, nblocks)
      {
        int bl = 0;
        for (int ib = ibtop; ib >= jb + nb; ib -= stride) {
          bl++;
          int ib2 = MIN(n, ib + pnb - 1), nb2 = ib2 - ib + 1;
          double* vr = &VRx(1, 1, bl);
          double* tr = &TRx(1, 1, bl);
          /* generation of the reflectors, ab2rht.f90:282-312 */
#pragma omp task depend(in : tokB22) depend(out : vr[0]) depend(out : tr[0]) firstprivate(bl, ib, ib2, nb2, vr, tr)
          {
            double* work = malloc(sizeof(double) * ((size_t)lwork + pnb + 64));
            lacpy(nb2, nb2, &IX(B, ldb, ib, ib), ldb, Bc, pnb);          /* :290 */
            gerqf(nb2, nb2, Bc, pnb, work, work + nb2, lwork - nb2);      /* :291 */
            if (nb2 > nb) {
              orgrq(nb2, nb2, nb2, Bc, pnb, work, work + pnb, lwork - nb2); /* :297 */
              gelq2(nb, nb2, Bc, pnb, work, work + nb);                   /* :298 */
              lacpy(nb, nb2, Bc, pnb, vr, nb);                             /* :299 */
              larft("F", "R", nb2, nb, vr, nb, work, tr, nb);              /* :302 */
            } else {
              larft("B", "R", nb2, nb2, Bc, pnb, work, tr, nb);            /* :308 */
              lacpy(nb2, nb2, Bc, pnb, vr, nb);                            /* :309 */
            }
            free(work);
          }
          /* lookahead update of B, ab2rht.f90:317-338 */
#pragma omp task depend(inout : tokB22) depend(in : tokB33) depend(in : vr[0]) depend(in : tr[0]) \
    firstprivate(bl, ib, ib2, nb2, vr, tr)
          {
            int c1 = MAX(1, ib - nb * (p - 1)), c2 = ib2;
            double* work = malloc(sizeof(double) * (size_t)(c2 - c1 + 1) * pnb);
            if (nb2 > nb) {
              larfb("R", "N", "F", "R", c2 - c1 + 1, nb2, nb, vr, nb, tr, nb, &IX(B, ldb, c1, ib), ldb, work,
                    c2 - c1 + 1); /* :327 */
              for (int j = ib; j <= ib + nb - 1; j++)
                for (int i = j + 1; i <= ib2; i++) IX(B, ldb, i, j) = 0.0; /* :329-333 */
            } else {
              larfb("R", "N", "B", "R", c2 - c1 + 1, nb2, nb2, vr, nb, tr, nb, &IX(B, ldb, c1, ib), ldb, work,
                    c2 - c1 + 1); /* :335 */
            }
            free(work);
          }
          /* update of the rest of B, ab2rht.f90:343-367 */
#pragma omp task depend(inout : tokB33) depend(in : vr[0]) depend(in : tr[0]) firstprivate(bl, ib, ib2, nb2, vr, tr)
          {
#pragma omp taskloop firstprivate(bl, ib, ib2, nb2, vr, tr)
            for (int i = 1; i <= ib; i += blocksize) {
              int c1 = i, c2 = MIN(i + blocksize - 1, MAX(1, ib - nb * (p - 1)) - 1);
              if (c2 >= c1) {
                double* work = malloc(sizeof(double) * (size_t)blocksize * pnb);
                if (nb2 > nb)
                  larfb("R", "N", "F", "R", c2 - c1 + 1, nb2, nb, vr, nb, tr, nb, &IX(B, ldb, c1, ib), ldb, work,
                        c2 - c1 + 1); /* :359 */
                else
                  larfb("R", "N", "B", "R", c2 - c1 + 1, nb2, nb2, vr, nb, tr, nb, &IX(B, ldb, c1, ib), ldb, work,
                        c2 - c1 + 1); /* :362 */
                free(work);
              }
            }
          }
        }
#pragma omp taskwait
      }
      if (time_components) {
#pragma omp taskwait
        double t1 = now_s();
        t_genright += t1 - t0;
        t0 = t1;
      }
      /* ---- apply right reflectors to A, ab2rht.f90:387-425 ---- */
#pragma omp task depend(inout : tokA) depend(in : tokVR) depend(in : tokTR) priority(1) firstprivate(jb, nblocks)
      {
#pragma omp taskloop firstprivate(jb, nblocks)
        for (int i = 1; i <= n; i += blocksize) {
          int r1 = i, r2 = MIN(i + blocksize - 1, n);
          double* work = malloc(sizeof(double) * (size_t)blocksize * pnb);
          int bl = 0;
          for (int ib = ibtop; ib >= jb + nb; ib -= stride) {
            bl++;
            int ib2 = MIN(n, ib + pnb - 1), nb2 = ib2 - ib + 1;
            if (nb2 > nb)
              larfb("R", "N", "F", "R", r2 - r1 + 1, nb2, nb, &VRx(1, 1, bl), nb, &TRx(1, 1, bl), nb,
                    &IX(A, lda, r1, ib), lda, work, r2 - r1 + 1); /* :412 */
            else
              larfb("R", "N", "B", "R", r2 - r1 + 1, nb2, nb2, &VRx(1, 1, bl), nb, &TRx(1, 1, bl), nb,
                    &IX(A, lda, r1, ib), lda, work, r2 - r1 + 1); /* :415 */
          }
          free(work);
        }
      }
      /* ---- apply right reflectors to Z, ab2rht.f90:430-467 ---- */
#pragma omp task depend(inout : tokZ) depend(in : tokVR) depend(in : tokTR) priority(1) firstprivate(jb, nblocks)
      {
#pragma omp taskloop firstprivate(jb, nblocks)
        for (int i = 1; i <= n; i += blocksize) {
          int r1 = i, r2 = MIN(i + blocksize - 1, n);
          double* work = malloc(sizeof(double) * (size_t)blocksize * pnb);
          int bl = 0;
          for (int ib = ibtop; ib >= jb + nb; ib -= stride) {
            bl++;
            int ib2 = MIN(n, ib + pnb - 1), nb2 = ib2 - ib + 1;
            if (nb2 > nb)
              larfb("R", "N", "F", "R", r2 - r1 + 1, nb2, nb, &VRx(1, 1, bl), nb, &TRx(1, 1, bl), nb,
                    &IX(Z, ldz, r1, ib), ldz, work, r2 - r1 + 1); /* :455 */
            else
              larfb("R", "N", "B", "R", r2 - r1 + 1, nb2, nb2, &VRx(1, 1, bl), nb, &TRx(1, 1, bl), nb,
                    &IX(Z, ldz, r1, ib), ldz, work, r2 - r1 + 1); /* :458 */
          }
          free(work);
        }
      }
      if (time_components) {
#pragma omp taskwait
        double t1 = now_s();
        t_mul += t1 - t0;
        t0 = t1;
      }
    }
#pragma omp taskwait
  }
#undef VLx
#undef VRx
#undef TLx
#undef TRx
  if (phase) {
    phase[0] = t_genleft;
    phase[1] = t_genright;
    phase[2] = t_mul;
  }
  free(VL);
  free(VR);
  free(TL);
  free(TR);
  free(Bc);
  return 0;
}

/* ======================================================================================
 * Stage 2: rht2ht_householder (src/rht2ht.f90:1346-2051)
 * phase[0..2] <- generation, lookahead, application times (rht2ht.f90:2044-2047)
 * ====================================================================================== */
int oracle_rht2ht_householder(int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z, int ldz,
                              int r, int nq, int time_components, double* phase) {
  if (init_lapack()) return -100;
  if (n < 1 || r < 1 || nq < 1) return -1;
  int nblk0 = (n - 1) / r;
  if ((n - 1) % r != 0) nblk0++; /* rht2ht.f90:1383-1384 */
  if (nblk0 < 1) nblk0 = 1;
  const int ldu = r + nq;
  const size_t usz = (size_t)ldu * nq * nblk0, tsz = (size_t)nq * nq * nblk0, tausz = (size_t)nq * nblk0;
  double* U = calloc(usz, sizeof(double));
  double* V = calloc(usz, sizeof(double));
  double* TU = calloc(tsz, sizeof(double));
  double* TV = calloc(tsz, sizeof(double));
  double* tauU = calloc(tausz, sizeof(double));
  double* tauV = calloc(tausz, sizeof(double));
  double* U2 = calloc(usz, sizeof(double));
  double* V2 = calloc(usz, sizeof(double));
  double* TU2 = calloc(tsz, sizeof(double));
  double* TV2 = calloc(tsz, sizeof(double));
  double* tauU2 = calloc(tausz, sizeof(double));
  double* tauV2 = calloc(tausz, sizeof(double));
  double* Bc = calloc((size_t)r * r, sizeof(double));
  const size_t wsz = (size_t)(r + nq) * (n + 64);
  double t_gen = 0, t_look = 0, t_app = 0, t0 = 0;
  char tokA, tokA22, tokB, tokB22, tokQ, tokZ, tokU, tokV, tokTU, tokTV, tokU2, tokV2, tokTU2, tokTV2;
#define Ux(i, j, b) U[((size_t)(i)-1) + ((size_t)(j)-1) * ldu + ((size_t)(b)-1) * ldu * nq]
#define Vx(i, j, b) V[((size_t)(i)-1) + ((size_t)(j)-1) * ldu + ((size_t)(b)-1) * ldu * nq]
#define U2x(i, j, b) U2[((size_t)(i)-1) + ((size_t)(j)-1) * ldu + ((size_t)(b)-1) * ldu * nq]
#define V2x(i, j, b) V2[((size_t)(i)-1) + ((size_t)(j)-1) * ldu + ((size_t)(b)-1) * ldu * nq]
#define TUx(i, j, b) TU[((size_t)(i)-1) + ((size_t)(j)-1) * nq + ((size_t)(b)-1) * nq * nq]
#define TVx(i, j, b) TV[((size_t)(i)-1) + ((size_t)(j)-1) * nq + ((size_t)(b)-1) * nq * nq]
#define TU2x(i, j, b) TU2[((size_t)(i)-1) + ((size_t)(j)-1) * nq + ((size_t)(b)-1) * nq * nq]
#define TV2x(i, j, b) TV2[((size_t)(i)-1) + ((size_t)(j)-1) * nq + ((size_t)(b)-1) * nq * nq]
#define tUx(i, b) tauU[((size_t)(i)-1) + ((size_t)(b)-1) * nq]
#define tVx(i, b) tauV[((size_t)(i)-1) + ((size_t)(b)-1) * nq]
#define tU2x(i, b) tauU2[((size_t)(i)-1) + ((size_t)(b)-1) * nq]
#define tV2x(i, b) tauV2[((size_t)(i)-1) + ((size_t)(b)-1) * nq]
#define Ax(i, j) IX(A, lda, i, j)
#define Bx(i, j) IX(B, ldb, i, j)
#define Bcx(i, j) IX(Bc, r, i, j)

#pragma omp parallel
#pragma omp single
  {
    const int blocksize = chunk_size(n);
    const char* dbg = getenv("PARAHT_ORACLE_STAGE2_LAST_JBLOCK"); /* debugging aid: stop after this group */
    const int last_jblock = dbg ? atoi(dbg) : n;
    for (int jblock = 1; jblock <= n - 2 && jblock <= last_jblock; jblock += nq) { /* rht2ht.f90:1417 */
      int nblocks = (n - jblock) / r;
      if ((n - jblock) % r != 0) nblocks++; /* :1420-1421 */
      if (time_components) {
#pragma omp taskwait
        t0 = now_s();
      }
      /* ---- generation: band-only chase of nq columns, rht2ht.f90:1433-1617 ---- */
#pragma omp task depend(inout : tokA) depend(inout : tokB) depend(out : tokU) depend(out : tokTU) depend(out : tokV) \
    depend(out : tokTV) priority(100) firstprivate(jblock, nblocks)
      {
        double* work = malloc(sizeof(double) * wsz);
        memset(U, 0, usz * sizeof(double)); /* :1442-1447 */
        memset(V, 0, usz * sizeof(double));
        memset(TU, 0, tsz * sizeof(double));
        memset(TV, 0, tsz * sizeof(double));
        memset(tauU, 0, tausz * sizeof(double));
        memset(tauV, 0, tausz * sizeof(double));
        for (int ic = 1; ic <= nq; ic++) { /* :1450 */
          int jc = jblock + ic - 1;
          int nb = MIN(r, n - jc);
          int istart = jblock + 1;
          if (jc + r <= n) /* :1466-1471 */
            for (int i = 1; i <= ic - 1; i++) larf("L", r, 1, &Ux(i, i, 1), 1, &tUx(i, 1), &Bx(jblock + i, jc + r), ldb, work);
          for (int i = 1; i <= ic - 1; i++) /* :1477-1482 */
            if (jc <= n) larf("L", MIN(r, n - jblock - i + 1), 1, &Ux(i, i, 1), 1, &tUx(i, 1), &Ax(jblock + i, jc), lda, work);
          if (nb < 2) continue; /* :1484 */
          larfg(nb, &Ax(jc + 1, jc), &Ax(jc + 2, jc), 1, &tUx(ic, 1)); /* :1487 */
          for (int i = 2; i <= nb; i++) {
            Ux(ic + i - 1, ic, 1) = Ax(jc + i, jc);
            Ax(jc + i, jc) = 0.0;
          }
          Ux(ic, ic, 1) = 1.0;
          larf("L", nb, nb, &Ux(ic, ic, 1), 1, &tUx(ic, 1), &Bx(jc + 1, jc + 1), ldb, work); /* :1495 */
          lacpy(nb, nb, &Bx(jc + 1, jc + 1), ldb, Bc, r);                                  /* :1499 */
          gerq2(nb, nb, Bc, r, work, work + nb);                                            /* :1500 */
          orgr2(nb, nb, nb, Bc, r, work, work + nb);                                        /* :1502 */
          larfg(nb, &Bcx(1, 1), &Bcx(1, 2), r, &tVx(ic, 1));                                /* :1504 */
          for (int i = 2; i <= nb; i++) Vx(ic + i - 1, ic, 1) = Bcx(1, i);
          Vx(ic, ic, 1) = 1.0;
          larf("R", MIN(n, jc + r + nb) - jc, nb, &Vx(ic, ic, 1), 1, &tVx(ic, 1), &Ax(jc + 1, jc + 1), lda, work); /* :1510 */
          larf("R", nb, nb, &Vx(ic, ic, 1), 1, &tVx(ic, 1), &Bx(jc + 1, jc + 1), ldb, work); /* :1513 */
          for (int i = 2; i <= nb; i++) Bx(jc + i, jc + 1) = 0.0;
          larf("R", jc - istart + 1, nb, &Vx(ic, ic, 1), 1, &tVx(ic, 1), &Ax(istart, jc + 1), lda, work); /* :1518 */
          larf("R", jc - istart + 1, nb, &Vx(ic, ic, 1), 1, &tVx(ic, 1), &Bx(istart, jc + 1), ldb, work); /* :1520 */
          /* chase, :1528-1594 */
          for (int jb = jc + 1; jb <= n; jb += r) {
            int ib = (jb - (jc + 1)) / r + 2;
            nb = MIN(r, n - jb - r + 1);
            istart = MAX(jblock + 1, jblock + 1 + (ib - 1) * r - (nq - ic) * r);
            if (jb + r + r - 1 <= n) /* :1539-1544 */
              for (int i = 1; i <= ic - 1; i++)
                larf("L", r, 1, &Ux(i, i, ib), 1, &tUx(i, ib), &Bx(jb + r - ic + i, jb + r + r - 1), ldb, work);
            for (int i = 1; i <= ic - 1; i++) /* :1550-1553 */
              if (jb + r - ic + i <= n)
                larf("L", MIN(r, n - (jb + r - ic + i) + 1), 1, &Ux(i, i, ib), 1, &tUx(i, ib), &Ax(jb + r - ic + i, jb),
                     lda, work);
            if (nb < 2) continue; /* :1555 */
            larfg(nb, &Ax(jb + r, jb), &Ax(jb + r + 1, jb), 1, &tUx(ic, ib)); /* :1558 */
            for (int i = 1; i <= nb - 1; i++) {
              Ux(ic + i, ic, ib) = Ax(jb + r + i, jb);
              Ax(jb + r + i, jb) = 0.0;
            }
            Ux(ic, ic, ib) = 1.0;
            larf("L", nb, nb, &Ux(ic, ic, ib), 1, &tUx(ic, ib), &Bx(jb + r, jb + r), ldb, work); /* :1566 */
            lacpy(nb, nb, &Bx(jb + r, jb + r), ldb, Bc, r);
            gerq2(nb, nb, Bc, r, work, work + nb);
            orgr2(nb, nb, nb, Bc, r, work, work + nb);
            larfg(nb, &Bcx(1, 1), &Bcx(1, 2), r, &tVx(ic, ib)); /* :1575 */
            for (int i = 2; i <= nb; i++) Vx(ic + i - 1, ic, ib) = Bcx(1, i);
            Vx(ic, ic, ib) = 1.0;
            larf("R", MIN(n, jb + 2 * r + nb - 1) - jb - r + 1, nb, &Vx(ic, ic, ib), 1, &tVx(ic, ib), &Ax(jb + r, jb + r),
                 lda, work); /* :1581 */
            larf("R", nb, nb, &Vx(ic, ic, ib), 1, &tVx(ic, ib), &Bx(jb + r, jb + r), ldb, work); /* :1584 */
            for (int i = 1; i <= nb - 1; i++) Bx(jb + r + i, jb + r) = 0.0;
            larf("R", jb + r - istart, nb, &Vx(ic, ic, ib), 1, &tVx(ic, ib), &Ax(istart, jb + r), lda, work); /* :1589 */
            larf("R", jb + r - istart, nb, &Vx(ic, ic, ib), 1, &tVx(ic, ib), &Bx(istart, jb + r), ldb, work); /* :1591 */
          }
        }
        for (int ib = nblocks; ib >= 1; ib--) { /* :1599-1603 */
          int jb = jblock + (ib - 1) * r;
          int nb = MIN(n - jb, r + nq);
          larft("F", "C", nb, MIN(nq, nb), &Ux(1, 1, ib), ldu, &tUx(1, ib), &TUx(1, 1, ib), nq);
        }
        for (int ib = nblocks; ib >= 1; ib--) { /* :1606-1610 */
          int jb = jblock + (ib - 1) * r;
          int nb = MIN(n - jb, r + nq);
          larft("F", "C", nb, MIN(nq, nb), &Vx(1, 1, ib), ldu, &tVx(1, ib), &TVx(1, 1, ib), nq);
        }
        free(work);
      }
      if (time_components) {
#pragma omp taskwait
        double t1 = now_s();
        t_gen += t1 - t0;
        t0 = t1;
      }
      /* ---- lookahead on B, rht2ht.f90:1630-1690 ---- */
#pragma omp task depend(inout : tokB22) depend(inout : tokB) depend(in : tokV) depend(in : tokTV) depend(in : tokU) \
    depend(in : tokTU) priority(100) firstprivate(jblock, nblocks)
      {
#pragma omp taskloop firstprivate(jblock, nblocks)
        for (int i = 1; i <= n; i += blocksize) { /* right, :1644-1661 */
          double* work = malloc(sizeof(double) * wsz);
          for (int ib = nblocks; ib >= 1; ib--) {
            int jb = jblock + (ib - 1) * r;
            for (int ic = 1; ic <= nq; ic++) {
              int istart = MAX(jblock + 1, jblock + 1 + (ib - 1) * r - nq * r - (nq - ic) * r);
              int istart2 = MAX(jblock + 1, jblock + 1 + (ib - 1) * r - (nq - ic) * r);
              int r1 = MAX(i, istart), r2 = MIN(i + blocksize - 1, istart2 - 1);
              if (r2 >= r1) larf("R", r2 - r1 + 1, MIN(r, n - jb - ic + 1), &Vx(ic, ic, ib), 1, &tVx(ic, ib), &Bx(r1, jb + ic), ldb, work);
            }
          }
          free(work);
        }
#pragma omp taskloop firstprivate(jblock, nblocks)
        for (int i = 1; i <= n; i += blocksize) { /* left, :1669-1684 */
          double* work = malloc(sizeof(double) * wsz);
          for (int ib = nblocks; ib >= 1; ib--) {
            int jb = jblock + (ib - 1) * r;
            int nb = MIN(n - jb, r + nq);
            int istop = MIN(n, jblock + (ib - 1) * r + r + nq - 1);
            int istop2 = MIN(n, jblock + (ib - 1) * r + r + nq + r * nq - 1);
            int c1 = MAX(istop + 1, i), c2 = MIN(istop2, i + blocksize - 1);
            if (c2 >= c1)
              larfb("L", "T", "F", "C", nb, c2 - c1 + 1, MIN(nq, nb), &Ux(1, 1, ib), ldu, &TUx(1, 1, ib), nq,
                    &Bx(jb + 1, c1), ldb, work, c2 - c1 + 1);
          }
          free(work);
        }
      }
      /* ---- lookahead on A, rht2ht.f90:1696-1772 ---- */
#pragma omp task depend(inout : tokA22) depend(inout : tokA) depend(in : tokV) depend(in : tokTV) depend(in : tokU) \
    depend(in : tokTU) priority(100) firstprivate(jblock, nblocks)
      {
#pragma omp taskloop firstprivate(jblock, nblocks)
        for (int i = 1; i <= n; i += blocksize) { /* right, :1710-1728 */
          double* work = malloc(sizeof(double) * wsz);
          for (int ib = nblocks; ib >= 1; ib--) {
            int jb = jblock + (ib - 1) * r;
            for (int ic = 1; ic <= nq; ic++) {
              int istart = MAX(jblock + 1, jblock + 1 + (ib - 1) * r - nq * r - (nq - ic) * r);
              int istart2 = MAX(jblock + 1, jblock + 1 + (ib - 1) * r - (nq - ic) * r);
              int r1 = MAX(i, istart), r2 = MIN(i + blocksize - 1, istart2 - 1);
              if (r2 >= r1) larf("R", r2 - r1 + 1, MIN(r, n - jb - ic + 1), &Vx(ic, ic, ib), 1, &tVx(ic, ib), &Ax(r1, jb + ic), lda, work);
            }
          }
          free(work);
        }
#pragma omp taskloop firstprivate(jblock, nblocks)
        for (int i = 1; i <= n; i += blocksize) { /* left, :1737-1765 */
          double* work = malloc(sizeof(double) * wsz);
          for (int ib = nblocks; ib >= 1; ib--) {
            int jb, nb, istop, istop2, c1, c2;
            if (ib == 1) {
              jb = jblock;
              nb = MIN(n - jb, r + nq);
              istop = MIN(n, jb + nq - 1);
              istop2 = MIN(n, jblock + (ib - 1) * r + r + nq + r * nq - 1);
              c1 = MAX(istop + 1, i);
              c2 = MIN(istop2, i + blocksize - 1);
              if (c2 >= c1)
                larfb("L", "T", "F", "C", nb, c2 - c1 + 1, MIN(nq, nb), &Ux(1, 1, ib), ldu, &TUx(1, 1, ib), nq,
                      &Ax(jb + 1, c1), lda, work, c2 - c1 + 1); /* :1748 */
            } else {
              jb = jblock + 1 + (ib - 2) * r;
              nb = MIN(n - jb - r + 1, r + nq);
              istop = MIN(n, jb + nq - 1);
              istop2 = MIN(n, jblock + (ib - 1) * r + r + nq + r * nq - 1);
              c1 = MAX(istop + 1, i);
              c2 = MIN(istop2, i + blocksize - 1);
              if (c2 >= c1)
                larfb("L", "T", "F", "C", nb, c2 - c1 + 1, MIN(nq, nb), &Ux(1, 1, ib), ldu, &TUx(1, 1, ib), nq,
                      &Ax(jb + r, c1), lda, work, c2 - c1 + 1); /* :1759 */
            }
          }
          free(work);
        }
      }
      if (time_components) {
#pragma omp taskwait
        double t1 = now_s();
        t_look += t1 - t0;
        t0 = t1;
      }
      /* ---- copy reflectors so the next generation can start, rht2ht.f90:1786-1797 ---- */
#pragma omp task depend(in : tokU) depend(in : tokV) depend(in : tokTU) depend(in : tokTV) depend(out : tokU2) \
    depend(out : tokV2) depend(out : tokTU2) depend(out : tokTV2) priority(100)
      {
        memcpy(U2, U, usz * sizeof(double));
        memcpy(V2, V, usz * sizeof(double));
        memcpy(TU2, TU, tsz * sizeof(double));
        memcpy(TV2, TV, tsz * sizeof(double));
        memcpy(tauV2, tauV, tausz * sizeof(double));
        memcpy(tauU2, tauU, tausz * sizeof(double));
      }
      /* ---- update B, rht2ht.f90:1803-1873 ---- */
#pragma omp task depend(inout : tokB22) depend(in : tokV2) depend(in : tokTV2) depend(in : tokU2) depend(in : tokTU2) \
    priority(1) firstprivate(jblock, nblocks)
      {
#pragma omp taskloop firstprivate(jblock, nblocks)
        for (int i = 1; i <= n; i += blocksize) { /* right, :1818-1844 */
          double* work = malloc(sizeof(double) * wsz);
          for (int ib = nblocks; ib >= 1; ib--) {
            int jb = jblock + (ib - 1) * r;
            int nb = MIN(n - jb, r + nq);
            int istart = MAX(jblock + 1, jblock + 1 + (ib - 1) * r - (2 * nq - 1) * r);
            if (i + blocksize - 1 >= istart) {
              int r1 = MAX(istart, i);
              for (int ic = 2; ic <= nq; ic++) {
                int istart2 = MAX(jblock + 1, jblock + 1 + (ib - 1) * r - nq * r - (nq - ic) * r);
                int r2 = MIN(i + blocksize - 1, istart2 - 1);
                if (r2 >= r1)
                  larf("R", r2 - r1 + 1, MIN(r, n - jb - ic + 1), &V2x(ic, ic, ib), 1, &tV2x(ic, ib), &Bx(r1, jb + ic), ldb, work);
              }
            }
            int r1 = i, r2 = MIN(i + blocksize - 1, istart - 1);
            larfb("R", "N", "F", "C", r2 - r1 + 1, nb, MIN(nq, nb), &V2x(1, 1, ib), ldu, &TV2x(1, 1, ib), nq, &Bx(r1, jb + 1),
                  ldb, work, r2 - r1 + 1); /* :1841 */
          }
          free(work);
        }
#pragma omp taskloop firstprivate(jblock, nblocks)
        for (int i = 1; i <= n; i += blocksize) { /* left, :1852-1866 */
          double* work = malloc(sizeof(double) * wsz);
          int c2 = MIN(n, i + blocksize - 1);
          for (int ib = nblocks; ib >= 1; ib--) {
            int jb = jblock + (ib - 1) * r;
            int nb = MIN(n - jb, r + nq);
            int istop = MIN(n, jblock + (ib - 1) * r + r + nq + r * nq - 1);
            int c1 = MAX(istop + 1, i);
            if (c2 >= c1)
              larfb("L", "T", "F", "C", nb, c2 - c1 + 1, MIN(nq, nb), &U2x(1, 1, ib), ldu, &TU2x(1, 1, ib), nq,
                    &Bx(jb + 1, c1), ldb, work, c2 - c1 + 1); /* :1862 */
          }
          free(work);
        }
      }
      /* ---- update A, rht2ht.f90:1880-1958 ---- */
#pragma omp task depend(inout : tokA22) depend(in : tokV2) depend(in : tokTV2) depend(in : tokU2) depend(in : tokTU2) \
    priority(1) firstprivate(jblock, nblocks)
      {
#pragma omp taskloop firstprivate(jblock, nblocks)
        for (int i = 1; i <= n; i += blocksize) { /* right, :1894-1920 */
          double* work = malloc(sizeof(double) * wsz);
          for (int ib = nblocks; ib >= 1; ib--) {
            int jb = jblock + (ib - 1) * r;
            int nb = MIN(n - jb, r + nq);
            int istart = MAX(jblock + 1, jblock + 1 + (ib - 1) * r - (2 * nq - 1) * r);
            if (i + blocksize - 1 >= istart) {
              int r1 = MAX(istart, i);
              for (int ic = 2; ic <= nq; ic++) {
                int istart2 = MAX(jblock + 1, jblock + 1 + (ib - 1) * r - (2 * nq - ic) * r);
                int r2 = MIN(i + blocksize - 1, istart2 - 1);
                if (r2 >= r1)
                  larf("R", r2 - r1 + 1, MIN(r, n - jb - ic + 1), &V2x(ic, ic, ib), 1, &tV2x(ic, ib), &Ax(r1, jb + ic), lda, work);
              }
            }
            int r1 = i, r2 = MIN(i + blocksize - 1, istart - 1);
            larfb("R", "N", "F", "C", r2 - r1 + 1, nb, MIN(nq, nb), &V2x(1, 1, ib), ldu, &TV2x(1, 1, ib), nq, &Ax(r1, jb + 1),
                  lda, work, r2 - r1 + 1); /* :1917 */
          }
          free(work);
        }
#pragma omp taskloop firstprivate(jblock, nblocks)
        for (int i = 1; i <= n; i += blocksize) { /* left, :1928-1951 */
          double* work = malloc(sizeof(double) * wsz);
          int c2 = MIN(n, i + blocksize - 1);
          for (int ib = nblocks; ib >= 1; ib--) {
            int istop = MIN(n, jblock + (ib - 1) * r + r + nq + r * nq - 1);
            int c1 = MAX(istop + 1, i);
            if (c2 >= c1) {
              if (ib == 1) {
                int jb = jblock;
                int nb = MIN(n - jb, r + nq);
                larfb("L", "T", "F", "C", nb, c2 - c1 + 1, MIN(nq, nb), &U2x(1, 1, ib), ldu, &TU2x(1, 1, ib), nq,
                      &Ax(jb + 1, c1), lda, work, c2 - c1 + 1); /* :1940 */
              } else {
                int jb = jblock + 1 + (ib - 2) * r;
                int nb = MIN(n - jb - r + 1, r + nq);
                larfb("L", "T", "F", "C", nb, c2 - c1 + 1, MIN(nq, nb), &U2x(1, 1, ib), ldu, &TU2x(1, 1, ib), nq,
                      &Ax(jb + r, c1), lda, work, c2 - c1 + 1); /* :1945 */
              }
            }
          }
          free(work);
        }
      }
      /* ---- update Q, rht2ht.f90:1964-1993 ---- */
#pragma omp task depend(inout : tokQ) depend(in : tokU2) depend(in : tokTU2) priority(1) firstprivate(jblock, nblocks)
      {
#pragma omp taskloop firstprivate(jblock, nblocks)
        for (int i = 1; i <= n; i += blocksize) {
          double* work = malloc(sizeof(double) * wsz);
          int r1 = i, r2 = MIN(n, i + blocksize - 1);
          for (int ib = nblocks; ib >= 1; ib--) {
            int jb = jblock + (ib - 1) * r;
            int nb = MIN(n - jb, r + nq - 1);
            larfb("R", "N", "F", "C", r2 - r1 + 1, nb, MIN(nq, nb), &U2x(1, 1, ib), ldu, &TU2x(1, 1, ib), nq, &IX(Q, ldq, r1, jb + 1),
                  ldq, work, r2 - r1 + 1); /* :1982 */
          }
          free(work);
        }
      }
      /* ---- update Z, rht2ht.f90:1998-2024 ---- */
#pragma omp task depend(inout : tokZ) depend(in : tokV2) depend(in : tokTV2) priority(1) firstprivate(jblock, nblocks)
      {
#pragma omp taskloop firstprivate(jblock, nblocks)
        for (int i = 1; i <= n; i += blocksize) {
          double* work = malloc(sizeof(double) * wsz);
          int r1 = i, r2 = MIN(n, i + blocksize - 1);
          for (int ib = nblocks; ib >= 1; ib--) {
            int jb = jblock + (ib - 1) * r;
            int nb = MIN(n - jb, r + nq);
            larfb("R", "N", "F", "C", r2 - r1 + 1, nb, MIN(nq, nb), &V2x(1, 1, ib), ldu, &TV2x(1, 1, ib), nq, &IX(Z, ldz, r1, jb + 1),
                  ldz, work, r2 - r1 + 1); /* :2015 */
          }
          free(work);
        }
      }
      if (time_components) {
#pragma omp taskwait
        double t1 = now_s();
        t_app += t1 - t0;
        t0 = t1;
      }
    }
#pragma omp taskwait
  }
  if (phase) {
    phase[0] = t_gen;
    phase[1] = t_look;
    phase[2] = t_app;
  }
  free(U); free(V); free(TU); free(TV); free(tauU); free(tauV);
  free(U2); free(V2); free(TU2); free(TV2); free(tauU2); free(tauV2); free(Bc);
  return 0;
}

/* ======================================================================================
 * rht2ht_householder_unblocked (src/rht2ht.f90:2053-2180): simple sequential chase with
 * immediate full updates; used as an independent stage-2 cross-check.
 * ====================================================================================== */
int oracle_rht2ht_unblocked(int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z, int ldz, int r) {
  if (init_lapack()) return -100;
  double* work = malloc(sizeof(double) * (size_t)(2 * r * n + 64));
  double* Bc = calloc((size_t)r * r, sizeof(double));
  double tau, temp;
  for (int jc = 1; jc <= n - 2; jc++) {
    int nb = MIN(r, n - jc);
    larfg(nb, &Ax(jc + 1, jc), &Ax(jc + 2, jc), 1, &tau); /* :2085 */
    temp = Ax(jc + 1, jc);
    Ax(jc + 1, jc) = 1.0;
    larf("L", nb, n - jc, &Ax(jc + 1, jc), 1, &tau, &Ax(jc + 1, jc + 1), lda, work);
    larf("L", nb, n - jc, &Ax(jc + 1, jc), 1, &tau, &Bx(jc + 1, jc + 1), ldb, work);
    larf("R", n, nb, &Ax(jc + 1, jc), 1, &tau, &IX(Q, ldq, 1, jc + 1), ldq, work);
    Ax(jc + 1, jc) = temp;
    for (int i = 2; i <= nb; i++) Ax(jc + i, jc) = 0.0;
    lacpy(nb, nb, &Bx(jc + 1, jc + 1), ldb, Bc, r); /* :2103 */
    gerq2(nb, nb, Bc, r, work, work + nb);
    orgr2(nb, nb, nb, Bc, r, work, work + nb);
    larfg(nb, &Bcx(1, 1), &Bcx(1, 2), r, &tau);
    Bcx(1, 1) = 1.0;
    larf("R", n, nb, &Bcx(1, 1), r, &tau, &Ax(1, jc + 1), lda, work);
    larf("R", jc + nb, nb, &Bcx(1, 1), r, &tau, &Bx(1, jc + 1), ldb, work);
    larf("R", n, nb, &Bcx(1, 1), r, &tau, &IX(Z, ldz, 1, jc + 1), ldz, work);
    for (int i = 2; i <= nb; i++) Bx(jc + i, jc + 1) = 0.0;
    for (int jb = jc + 1; jb <= n - r; jb += r) { /* :2129 */
      nb = MIN(r, n - jb - r + 1);
      larfg(nb, &Ax(jb + r, jb), &Ax(jb + r + 1, jb), 1, &tau);
      temp = Ax(jb + r, jb);
      Ax(jb + r, jb) = 1.0;
      larf("L", nb, n - jb, &Ax(jb + r, jb), 1, &tau, &Ax(jb + r, jb + 1), lda, work);
      larf("L", nb, n - jb - r + 1, &Ax(jb + r, jb), 1, &tau, &Bx(jb + r, jb + r), ldb, work);
      larf("R", n, nb, &Ax(jb + r, jb), 1, &tau, &IX(Q, ldq, 1, jb + r), ldq, work);
      Ax(jb + r, jb) = temp;
      for (int i = 1; i <= nb - 1; i++) Ax(jb + r + i, jb) = 0.0;
      lacpy(nb, nb, &Bx(jb + r, jb + r), ldb, Bc, r);
      gerq2(nb, nb, Bc, r, work, work + nb);
      orgr2(nb, nb, nb, Bc, r, work, work + nb);
      larfg(nb, &Bcx(1, 1), &Bcx(1, 2), r, &tau);
      Bcx(1, 1) = 1.0;
      larf("R", n, nb, &Bcx(1, 1), r, &tau, &Ax(1, jb + r), lda, work);
      larf("R", jb + r + nb - 1, nb, &Bcx(1, 1), r, &tau, &Bx(1, jb + r), ldb, work);
      larf("R", n, nb, &Bcx(1, 1), r, &tau, &IX(Z, ldz, 1, jb + r), ldz, work);
      for (int i = 1; i <= nb - 1; i++) Bx(jb + r + i, jb + r) = 0.0;
    }
  }
  free(work);
  free(Bc);
  return 0;
}

/* ======================================================================================
 * rht2ht_givens (src/rht2ht.f90:696-1344): stage 2 with Givens rotations.  The bulge chase
 * reduces each column with nb-1 rotations from the left (dlartg/drot) and removes the single
 * subdiagonal fill they leave in B with nb-1 rotations from the right, so no RQ is needed; the
 * rotations of a group are accumulated into (r+nq) x (r+nq) orthogonal matrices U(ib), V(ib)
 * per block (:970-1003), and the lookahead and delayed updates apply those with dgemm (plus the
 * staircase rotations that precede a block's full update, :1018-1062, :1246-1274).
 *
 * Restated in the reference's task order (mb = 1, so the multi-block branch :1200-1243 is not
 * taken; a valid schedule of the reference's task graph, whose tasks touch disjoint data or are
 * ordered by their depend clauses).  The U2/V2/CV2/SV2 copies (:1158-1168) only let generation
 * k+1 overlap updates k in the reference; run in order, the originals serve.
 *
 * Deliberate deviation: the reference's right rotations on B in the lookahead (:1025-1029) and
 * the delayed update (:1252-1256) run over ig = r-1..1 where the A loops use min(r-1, n-jb-ic);
 * for the last block of a group that reaches columns beyond n, with the identity rotations
 * (c = 1, s = 0) left there by the generation.  The oracle uses the A loops' bound for B too:
 * the rotations skipped are exactly those identities (checked), and no column beyond n is read.
 * ====================================================================================== */
static void rot(lint n, double* x, lint incx, double* y, lint incy, double c, double s) {
  if (n <= 0) return;
  LP->drot(&n, x, &incx, y, &incy, &c, &s);
}
static void lartg(double f, double g, double* c, double* s, double* r) { LP->dlartg(&f, &g, c, s, r); }

int oracle_rht2ht_givens(int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z, int ldz, int r,
                         int nq) {
  if (init_lapack()) return -100;
  if (n < 3) return 0;
  const int ldu = r + nq;
  int nblk0 = (n - 1) / r + ((n - 1) % r != 0);
  double* U = malloc(sizeof(double) * (size_t)ldu * ldu * nblk0);
  double* V = malloc(sizeof(double) * (size_t)ldu * ldu * nblk0);
  double* CU = malloc(sizeof(double) * (size_t)ldu * nq * nblk0);
  double* SU = malloc(sizeof(double) * (size_t)ldu * nq * nblk0);
  double* CV = malloc(sizeof(double) * (size_t)ldu * nq * nblk0);
  double* SV = malloc(sizeof(double) * (size_t)ldu * nq * nblk0);
  double* work = malloc(sizeof(double) * (size_t)(r + nq) * n);
  if (!U || !V || !CU || !SU || !CV || !SV || !work) return -101;
  const double one = 1.0, zero = 0.0;
  int bad_skip = 0;
#define RX(M, i, ic, ib) (M)[((size_t)(i)-1) + ((size_t)(ic)-1) * ldu + ((size_t)(ib)-1) * ldu * nq]
#define GX(M, i, j, ib) (M)[((size_t)(i)-1) + ((size_t)(j)-1) * ldu + ((size_t)(ib)-1) * ldu * ldu]
  lint lu = ldu;
  for (int jblock = 1; jblock <= n - 2; jblock += nq) { /* :766 */
    const int nblocks = (n - jblock) / r + ((n - jblock) % r != 0);
    /* ---- generation: rotations, updating only a band of A and B (:776-960) ---- */
    for (size_t e = 0; e < (size_t)ldu * nq * nblk0; e++) {
      CU[e] = 1.0;
      CV[e] = 1.0;
      SU[e] = 0.0;
      SV[e] = 0.0;
    }
    for (int ic = 1; ic <= nq; ic++) {
      const int jc = jblock + ic - 1;
      int nb = MIN(r, n - jc);
      int istart = jblock + 1;
      if (jc + r <= n) /* :806-814 */
        for (int i = 1; i <= ic - 1; i++)
          for (int ig = r - 1; ig >= 1; ig--)
            rot(1, &Bx(jblock + i - 1 + ig, jc + r), ldb, &Bx(jblock + i + ig, jc + r), ldb, RX(CU, i + ig - 1, i, 1),
                RX(SU, i + ig - 1, i, 1));
      for (int i = 1; i <= ic - 1; i++) /* :820-828 */
        if (jc <= n)
          for (int ig = MIN(r - 1, n - (jblock + i)); ig >= 1; ig--)
            rot(1, &Ax(jblock + i - 1 + ig, jc), lda, &Ax(jblock + i + ig, jc), lda, RX(CU, i + ig - 1, i, 1),
                RX(SU, i + ig - 1, i, 1));
      if (nb < 2) continue;
      double temp;
      for (int ig = nb - 1; ig >= 1; ig--) { /* :833-838 */
        lartg(Ax(jc + ig, jc), Ax(jc + ig + 1, jc), &RX(CU, ic + ig - 1, ic, 1), &RX(SU, ic + ig - 1, ic, 1), &temp);
        Ax(jc + ig, jc) = temp;
        Ax(jc + ig + 1, jc) = 0.0;
      }
      for (int ig = nb - 1; ig >= 1; ig--) /* :840-843 */
        rot(nb, &Bx(jc + ig, jc + 1), ldb, &Bx(jc + ig + 1, jc + 1), ldb, RX(CU, ic + ig - 1, ic, 1),
            RX(SU, ic + ig - 1, ic, 1));
      for (int ig = nb - 1; ig >= 1; ig--) { /* :846-854 */
        lartg(Bx(jc + ig + 1, jc + ig + 1), Bx(jc + ig + 1, jc + ig), &RX(CV, ic + ig - 1, ic, 1),
              &RX(SV, ic + ig - 1, ic, 1), &temp);
        Bx(jc + ig + 1, jc + ig + 1) = temp;
        Bx(jc + ig + 1, jc + ig) = 0.0;
        rot(ig, &Bx(jc + 1, jc + ig + 1), 1, &Bx(jc + 1, jc + ig), 1, RX(CV, ic + ig - 1, ic, 1),
            RX(SV, ic + ig - 1, ic, 1));
      }
      for (int ig = nb - 1; ig >= 1; ig--) /* :856-859 */
        rot(MIN(n, jc + r + nb) - jc, &Ax(jc + 1, jc + ig + 1), 1, &Ax(jc + 1, jc + ig), 1,
            RX(CV, ic + ig - 1, ic, 1), RX(SV, ic + ig - 1, ic, 1));
      for (int ig = nb - 1; ig >= 1; ig--) /* :862-865 */
        rot(jc - istart + 1, &Bx(istart, jc + ig + 1), 1, &Bx(istart, jc + ig), 1, RX(CV, ic + ig - 1, ic, 1),
            RX(SV, ic + ig - 1, ic, 1));
      for (int ig = nb - 1; ig >= 1; ig--) /* :867-870 */
        rot(jc - istart + 1, &Ax(istart, jc + ig + 1), 1, &Ax(istart, jc + ig), 1, RX(CV, ic + ig - 1, ic, 1),
            RX(SV, ic + ig - 1, ic, 1));
      for (int jb = jc + 1; jb <= n; jb += r) { /* :879 chase the fill down */
        const int ib = (jb - (jc + 1)) / r + 2;
        nb = MIN(r, n - jb - r + 1);
        istart = MAX(jblock + 1, jblock + 1 + (ib - 1) * r - (nq - ic) * r);
        if (jb + r + r - 1 <= n) /* :892-900 */
          for (int i = 1; i <= ic - 1; i++)
            for (int ig = r - 1; ig >= 1; ig--)
              rot(1, &Bx(jb + r - ic + i + ig - 1, jb + r + r - 1), ldb, &Bx(jb + r - ic + i + ig, jb + r + r - 1), ldb,
                  RX(CU, i + ig - 1, i, ib), RX(SU, i + ig - 1, i, ib));
        for (int i = 1; i <= ic - 1; i++) /* :906-914 */
          if (jb + r - ic + i <= n)
            for (int ig = MIN(r, n - (jb + r - ic + i) + 1) - 1; ig >= 1; ig--)
              rot(1, &Ax(jb + r - ic + i + ig - 1, jb), lda, &Ax(jb + r - ic + i + ig, jb), lda,
                  RX(CU, i + ig - 1, i, ib), RX(SU, i + ig - 1, i, ib));
        if (nb < 2) continue;
        for (int ig = nb - 1; ig >= 1; ig--) { /* :919-924 */
          lartg(Ax(jb + r - 1 + ig, jb), Ax(jb + r + ig, jb), &RX(CU, ic + ig - 1, ic, ib), &RX(SU, ic + ig - 1, ic, ib),
                &temp);
          Ax(jb + ig + r - 1, jb) = temp;
          Ax(jb + ig + r, jb) = 0.0;
        }
        for (int ig = nb - 1; ig >= 1; ig--) /* :926-929 */
          rot(nb, &Bx(jb + r - 1 + ig, jb + r), ldb, &Bx(jb + ig + r, jb + r), ldb, RX(CU, ic + ig - 1, ic, ib),
              RX(SU, ic + ig - 1, ic, ib));
        for (int ig = nb - 1; ig >= 1; ig--) { /* :932-940 */
          lartg(Bx(jb + r + ig, jb + r + ig), Bx(jb + r + ig, jb + r + ig - 1), &RX(CV, ic + ig - 1, ic, ib),
                &RX(SV, ic + ig - 1, ic, ib), &temp);
          Bx(jb + r + ig, jb + r + ig) = temp;
          Bx(jb + r + ig, jb + r + ig - 1) = 0.0;
          rot(ig, &Bx(jb + r, jb + r + ig), 1, &Bx(jb + r, jb + r + ig - 1), 1, RX(CV, ic + ig - 1, ic, ib),
              RX(SV, ic + ig - 1, ic, ib));
        }
        for (int ig = nb - 1; ig >= 1; ig--) /* :942-945 */
          rot(MIN(n, jb + 2 * r + nb - 1) - (jb + r) + 1, &Ax(jb + r, jb + r + ig), 1, &Ax(jb + r, jb + r + ig - 1), 1,
              RX(CV, ic + ig - 1, ic, ib), RX(SV, ic + ig - 1, ic, ib));
        for (int ig = nb - 1; ig >= 1; ig--) /* :948-951 */
          rot(jb + r - istart, &Bx(istart, jb + r + ig), 1, &Bx(istart, jb + r + ig - 1), 1,
              RX(CV, ic + ig - 1, ic, ib), RX(SV, ic + ig - 1, ic, ib));
        for (int ig = nb - 1; ig >= 1; ig--) /* :953-956 */
          rot(jb + r - istart, &Ax(istart, jb + r + ig), 1, &Ax(istart, jb + r + ig - 1), 1,
              RX(CV, ic + ig - 1, ic, ib), RX(SV, ic + ig - 1, ic, ib));
      }
    }
    /* ---- accumulate the rotations into U(ib), V(ib) (:970-1003) ---- */
    for (int ib = 1; ib <= nblocks; ib++) {
      LP->dlaset("A", &lu, &lu, &zero, &one, &GX(U, 1, 1, ib), &lu, 1);
      for (int ic = 1; ic <= nq; ic++)
        for (int ig = r - 1; ig >= 1; ig--)
          rot(ldu, &GX(U, 1, ic - 1 + ig, ib), 1, &GX(U, 1, ic + ig, ib), 1, RX(CU, ic + ig - 1, ic, ib),
              RX(SU, ic + ig - 1, ic, ib));
      LP->dlaset("A", &lu, &lu, &zero, &one, &GX(V, 1, 1, ib), &lu, 1);
      for (int ic = 1; ic <= nq; ic++)
        for (int ig = r - 1; ig >= 1; ig--)
          rot(ldu, &GX(V, 1, ic + ig, ib), 1, &GX(V, 1, ic + ig - 1, ib), 1, RX(CV, ic + ig - 1, ic, ib),
              RX(SV, ic + ig - 1, ic, ib));
    }
    /* right rotations of block ib on rows [lo, hi) of X (the lookahead :1018-1029, :1074-1087
     * and the delayed update's staircase :1246-1257, :1289-1296); columns beyond n are not touched */
#define STAIR(X, ldx, ib, lo_of_ic, hi_of_ic)                                                              \
  do {                                                                                                     \
    const int jb_ = jblock + ((ib)-1) * r;                                                                 \
    for (int ic = 1; ic <= nq; ic++) {                                                                     \
      const int lo_ = (lo_of_ic), hi_ = (hi_of_ic);                                                        \
      if (hi_ <= lo_) continue;                                                                            \
      for (int ig = r - 1; ig >= 1; ig--) {                                                                \
        if (jb_ + ic + ig > n) {                                                                           \
          if (RX(CV, ic + ig - 1, ic, (ib)) != 1.0 || RX(SV, ic + ig - 1, ic, (ib)) != 0.0) bad_skip = 1; \
          continue;                                                                                        \
        }                                                                                                  \
        rot(hi_ - lo_, &IX(X, ldx, lo_, jb_ + ic + ig), 1, &IX(X, ldx, lo_, jb_ + ic + ig - 1), 1,         \
            RX(CV, ic + ig - 1, ic, (ib)), RX(SV, ic + ig - 1, ic, (ib)));                                 \
      }                                                                                                    \
    }                                                                                                      \
  } while (0)
    /* ---- lookahead on B (:1008-1049) ---- */
    for (int ib = nblocks; ib >= 1; ib--)
      STAIR(B, ldb, ib, MAX(jblock + 1, jblock + 1 + (ib - 1) * r - nq * r - (nq - ic) * r),
            MAX(jblock + 1, jblock + 1 + (ib - 1) * r - (nq - ic) * r));
    for (int ib = nblocks; ib >= 1; ib--) {
      const int jb = jblock + (ib - 1) * r, nb = MIN(n - jb, r + nq);
      const int istop = MIN(n, jblock + (ib - 1) * r + r + nq - 1);
      const int istop2 = MIN(n, jblock + (ib - 1) * r + r + nq + r * nq - 1);
      if (istop2 > istop) {
        lint m = nb, nn = istop2 - istop, lw = nb, lb = ldb;
        LP->dgemm("T", "N", &m, &nn, &m, &one, &GX(U, 1, 1, ib), &lu, &Bx(jb + 1, istop + 1), &lb, &zero, work, &lw, 1,
                  1);
        lacpy(nb, istop2 - istop, work, nb, &Bx(jb + 1, istop + 1), ldb);
      }
    }
    /* ---- lookahead on A (:1065-1131) ---- */
    for (int ib = nblocks; ib >= 1; ib--)
      STAIR(A, lda, ib, MAX(jblock + 1, jblock + 1 + (ib - 1) * r - nq * r - (nq - ic) * r),
            MAX(jblock + 1, jblock + 1 + (ib - 1) * r - (nq - ic) * r));
    for (int ib = nblocks; ib >= 1; ib--) {
      int jb, nb, row0;
      if (ib == 1) {
        jb = jblock;
        nb = MIN(n - jb, r + nq);
        row0 = jb + 1;
      } else {
        jb = jblock + 1 + (ib - 2) * r;
        nb = MIN(n - jb - r + 1, r + nq);
        row0 = jb + r;
      }
      const int istop = MIN(n, jb + nq - 1);
      const int istop2 = MIN(n, jblock + (ib - 1) * r + r + nq + r * nq - 1);
      if (istop2 > istop && nb > 0) {
        lint m = nb, nn = istop2 - istop, lw = nb, la = lda;
        LP->dgemm("T", "N", &m, &nn, &m, &one, &GX(U, 1, 1, ib), &lu, &Ax(row0, istop + 1), &la, &zero, work, &lw, 1,
                  1);
        lacpy(nb, istop2 - istop, work, nb, &Ax(row0, istop + 1), lda);
      }
    }
    /* ---- delayed update of B (:1173-1283): right (staircase rotations, then dgemm on rows
     * 1..istart-1), then left ---- */
    for (int ib = nblocks; ib >= 1; ib--) {
      const int jb = jblock + (ib - 1) * r, nb = MIN(n - jb, r + nq);
      const int istart = MAX(jblock + 1, jblock + 1 + (ib - 1) * r - (2 * nq - 1) * r);
      STAIR(B, ldb, ib, istart, MAX(jblock + 1, jblock + 1 + (ib - 1) * r - nq * r - (nq - ic) * r));
      if (istart - 1 >= 1) {
        lint m = istart - 1, nn = nb, lb = ldb, lw = istart - 1;
        LP->dgemm("N", "N", &m, &nn, &nn, &one, &Bx(1, jb + 1), &lb, &GX(V, 1, 1, ib), &lu, &zero, work, &lw, 1, 1);
        lacpy(istart - 1, nb, work, istart - 1, &Bx(1, jb + 1), ldb);
      }
    }
    for (int ib = nblocks; ib >= 1; ib--) {
      const int jb = jblock + (ib - 1) * r, nb = MIN(n - jb, r + nq);
      const int istop = MIN(n, jblock + (ib - 1) * r + r + nq + r * nq - 1);
      if (n > istop) {
        lint m = nb, nn = n - istop, lw = nb, lb = ldb;
        LP->dgemm("T", "N", &m, &nn, &m, &one, &GX(U, 1, 1, ib), &lu, &Bx(jb + 1, istop + 1), &lb, &zero, work, &lw, 1,
                  1);
        lacpy(nb, n - istop, work, nb, &Bx(jb + 1, istop + 1), ldb);
      }
    }
    /* ---- delayed update of A (:1290-1334) ---- */
    for (int ib = nblocks; ib >= 1; ib--) {
      const int jb = jblock + (ib - 1) * r, nb = MIN(n - jb, r + nq);
      const int istart = MAX(jblock + 1, jblock + 1 + (ib - 1) * r - (2 * nq - 1) * r);
      STAIR(A, lda, ib, istart, MAX(jblock + 1, jblock + 1 + (ib - 1) * r - (2 * nq - ic) * r));
      if (istart - 1 >= 1) {
        lint m = istart - 1, nn = nb, la = lda, lw = istart - 1;
        LP->dgemm("N", "N", &m, &nn, &nn, &one, &Ax(1, jb + 1), &la, &GX(V, 1, 1, ib), &lu, &zero, work, &lw, 1, 1);
        lacpy(istart - 1, nb, work, istart - 1, &Ax(1, jb + 1), lda);
      }
    }
    for (int ib = nblocks; ib >= 1; ib--) {
      int jb, nb, row0;
      if (ib == 1) {
        jb = jblock;
        nb = MIN(n - jb, r + nq);
        row0 = jb + 1;
      } else {
        jb = jblock + 1 + (ib - 2) * r;
        nb = MIN(n - jb - r + 1, r + nq);
        row0 = jb + r;
      }
      const int istop = MIN(n, jblock + (ib - 1) * r + r + nq + r * nq - 1);
      if (n > istop && nb > 0) {
        lint m = nb, nn = n - istop, lw = nb, la = lda;
        LP->dgemm("T", "N", &m, &nn, &m, &one, &GX(U, 1, 1, ib), &lu, &Ax(row0, istop + 1), &la, &zero, work, &lw, 1,
                  1);
        lacpy(nb, n - istop, work, nb, &Ax(row0, istop + 1), lda);
      }
    }
    /* ---- Q and Z (:1340-1366 of the task list: Q(:, jb+1:jb+nb) <- Q(:, ...) U(ib)) ---- */
    for (int ib = nblocks; ib >= 1; ib--) {
      const int jb = jblock + (ib - 1) * r, nb = MIN(n - jb, r + nq);
      lint m = n, nn = nb, lqq = ldq, lzz = ldz, lw = n;
      LP->dgemm("N", "N", &m, &nn, &nn, &one, &IX(Q, ldq, 1, jb + 1), &lqq, &GX(U, 1, 1, ib), &lu, &zero, work, &lw, 1,
                1);
      lacpy(n, nb, work, n, &IX(Q, ldq, 1, jb + 1), ldq);
      LP->dgemm("N", "N", &m, &nn, &nn, &one, &IX(Z, ldz, 1, jb + 1), &lzz, &GX(V, 1, 1, ib), &lu, &zero, work, &lw, 1,
                1);
      lacpy(n, nb, work, n, &IX(Z, ldz, 1, jb + 1), ldz);
    }
#undef STAIR
  }
#undef RX
#undef GX
  free(U);
  free(V);
  free(CU);
  free(SU);
  free(CV);
  free(SV);
  free(work);
  return bad_skip ? -102 : 0;
}

/* ======================================================================================
 * LAPACK baselines and checks used by the reference driver (src/profilereduction.f90).
 * ====================================================================================== */

/* profilereduction.f90:156: dgghd3('V','V',n,1,n,...) */
int oracle_dgghd3(int n, double* A, int lda, double* B, int ldb, double* Q, int ldq, double* Z, int ldz) {
  if (init_lapack()) return -100;
  lint nn = n, one = 1, info = 0, lwork = -1;
  lint la = lda, lb = ldb, lq = ldq, lz = ldz;
  double q;
  LP->dgghd3("V", "V", &nn, &one, &nn, A, &la, B, &lb, Q, &lq, Z, &lz, &q, &lwork, &info, 1, 1);
  lwork = MAX((lint)q, 1);
  double* work = malloc(sizeof(double) * lwork);
  LP->dgghd3("V", "V", &nn, &one, &nn, A, &la, B, &lb, Q, &lq, Z, &lz, work, &lwork, &info, 1, 1);
  free(work);
  return info;
}

/* dgghd3 with the caller's compq/compz and ilo/ihi (LAPACK's own interface), the reference result
 * for the library's DGGHD3-compatible entry in the tests. */
int oracle_dgghd3_range(char compq, char compz, int n, int ilo, int ihi, double* A, int lda, double* B, int ldb,
                        double* Q, int ldq, double* Z, int ldz) {
  if (init_lapack()) return -100;
  lint nn = n, lo = ilo, hi = ihi, info = 0, lwork = -1;
  lint la = lda, lb = ldb, lq = ldq, lz = ldz;
  char cq[2] = {compq, 0}, cz[2] = {compz, 0};
  double q;
  LP->dgghd3(cq, cz, &nn, &lo, &hi, A, &la, B, &lb, Q, &lq, Z, &lz, &q, &lwork, &info, 1, 1);
  lwork = MAX((lint)q, 1);
  double* work = malloc(sizeof(double) * lwork);
  LP->dgghd3(cq, cz, &nn, &lo, &hi, A, &la, B, &lb, Q, &lq, Z, &lz, work, &lwork, &info, 1, 1);
  free(work);
  return info;
}

/* Generalized eigenvalues of an HT pencil via DHGEQZ('E','N','N') (no Schur vectors). */
int oracle_dhgeqz_eigs(int n, double* H, int ldh, double* T, int ldt, double* alphar, double* alphai, double* beta) {
  if (init_lapack()) return -100;
  lint nn = n, one = 1, info = 0, lwork = -1, lh = ldh, lt = ldt, ldq = 1;
  double q, dq = 0, dz = 0;
  LP->dhgeqz("E", "N", "N", &nn, &one, &nn, H, &lh, T, &lt, alphar, alphai, beta, &dq, &ldq, &dz, &ldq, &q, &lwork,
             &info, 1, 1, 1);
  lwork = MAX((lint)q, n);
  double* work = malloc(sizeof(double) * lwork);
  LP->dhgeqz("E", "N", "N", &nn, &one, &nn, H, &lh, T, &lt, alphar, alphai, beta, &dq, &ldq, &dz, &ldq, work, &lwork,
             &info, 1, 1, 1);
  free(work);
  return info;
}

/* profilereduction.f90:117-123: B <- R factor of QR(B) (dgeqrf, zero below the diagonal). */
int oracle_triangularize(int n, double* B, int ldb) {
  if (init_lapack()) return -100;
  lint nn = n, lb = ldb, info = 0, lwork = -1;
  double q;
  double* tau = malloc(sizeof(double) * n);
  LP->dgeqrf(&nn, &nn, B, &lb, tau, &q, &lwork, &info);
  lwork = MAX((lint)q, n);
  double* work = malloc(sizeof(double) * lwork);
  LP->dgeqrf(&nn, &nn, B, &lb, tau, work, &lwork, &info);
  for (int j = 1; j <= n; j++)
    for (int i = j + 1; i <= n; i++) Bx(i, j) = 0.0;
  free(work);
  free(tau);
  return info;
}

/* profilereduction.f90:165-174: ||Q^T A0 Z - H||_F / ||A0||_F with profilereduction's own dgemm/dlange calls. */
double oracle_backward_error(int n, const double* Q, int ldq, const double* A0, int lda0, const double* Z, int ldz,
                             const double* H, int ldh) {
  if (init_lapack()) return -1.0;
  lint nn = n, lq = ldq, la = lda0, lz = ldz, ln = n;
  double one = 1.0, zero = 0.0, mone = -1.0;
  double* C = malloc(sizeof(double) * (size_t)n * n);
  double* R = malloc(sizeof(double) * (size_t)n * n);
  for (int j = 0; j < n; j++) memcpy(R + (size_t)j * n, H + (size_t)j * ldh, sizeof(double) * n);
  LP->dgemm("T", "N", &nn, &nn, &nn, &one, Q, &lq, A0, &la, &zero, C, &ln, 1, 1);
  LP->dgemm("N", "N", &nn, &nn, &nn, &one, C, &ln, Z, &lz, &mone, R, &ln, 1, 1);
  double nrm0 = LP->dlange("F", &nn, &nn, A0, &la, NULL, 1);
  double nrm = LP->dlange("F", &nn, &nn, R, &ln, NULL, 1);
  free(C);
  free(R);
  return nrm / nrm0;
}
#undef Ux
#undef Vx
#undef Ax
#undef Bx
#undef Bcx

/*
 * CPU oracle for the blocked matrix multiply C := beta*C + alpha*A*B.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker that the GPU path is
 * compared against, and the CPU baseline that the benchmark times beside it.
 * Nothing in the shipped GPU library links, loads or calls it.
 *
 * It restates, in portable C, the reference's Goto composition and its BLIS
 * Haswell microkernels, keeping their blocking and their per-element rounding
 * order so that results are bit-identical to the reference's own kernels:
 *
 *   loop nest  PartN(NC) -> PartK(KC) -> PackB -> PartM(MC) -> PackA
 *              -> ParallelN(NR, all threads) -> KernelNM(MR x NR)
 *     src/exper/l3_packing.rs:58-66     (composition, NC=3000 KC=192 MC=120)
 *     src/composables/part.rs:7-120     (PartM/PartN/PartK; PartK sets the
 *                                        C scalar to 1 after the first k slab,
 *                                        part.rs:96-110)
 *     src/composables/pack.rs:51-133    (panel copiers; layouts p[y*NR+i] for
 *                                        B panels, p[x*MR+i] for A panels)
 *     src/composables/pack.rs:328-351, 383-406 (barrier, pack, barrier)
 *     src/composables/parallel_range.rs:130-154 (ParallelN range split)
 *     src/kern/kernel_nm.rs:31-106      (jr/ir loops; full tiles call the
 *                                        microkernel on C; edge tiles compute
 *                                        tmp with beta=0 then c = tmp + beta*c
 *                                        as separate multiply and add)
 *   microkernel  ukernels/bli_gemm_haswell_asm_d6x8.c
 *     :725-885   acc = fma(a_p, b_p, acc) sequentially over p from acc = 0
 *     :889-910   acc *= alpha
 *     :920-935   beta == 0 (vucomisd: also taken for NaN beta) stores acc
 *     :939-1074  otherwise c = fma(beta, c, acc), row- or general-stored
 *   and bli_sgemm_haswell_asm_6x16 (same file, :77-640) for f32.
 *
 * Differences from the reference that do not change any valid output:
 *   - edge panels are zero-filled; the reference copies PW/PH elements past
 *     the matrix edge (out-of-bounds reads) and discards those lanes;
 *   - pack buffers are sized in elements * sizeof(T) (the reference passes an
 *     element count where bytes are expected, column_panel.rs:277).
 *
 * A caller may plug in another microkernel with the BLIS signature (the
 * reference's own asm kernel, compiled from its sources into oracle/_ref on
 * x86-64 hosts) through the `ukr` argument.
 *
 * Also here: a double-double (about 106-bit) accumulated GEMM used as the
 * high-accuracy oracle for error measurements, the componentwise magnitude
 * |alpha||A||B| + |beta||C|, and the reference's Freivalds residual check
 * (src/util.rs:55-85).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef int64_t dim_t;
typedef int64_t inc_t;

typedef void (*dukr_t)(dim_t, double*, double*, double*, double*, double*, inc_t, inc_t, void*, void*);
typedef void (*sukr_t)(dim_t, float*, float*, float*, float*, float*, inc_t, inc_t, void*, void*);

/* ------------------------------------------------------------------------ */
/* Portable microkernels with the reference's rounding order.                */
/* ------------------------------------------------------------------------ */

#define DMR 6
#define DNR 8
#define SMR 6
#define SNR 16

void oracle_ukr_d6x8(dim_t k, double* alpha, double* a, double* b, double* beta, double* c, inc_t rs_c,
                     inc_t cs_c, void* data, void* cntx) {
  (void)data;
  (void)cntx;
  double acc[DMR][DNR];
  for (int i = 0; i < DMR; i++)
    for (int j = 0; j < DNR; j++) acc[i][j] = 0.0;
  for (dim_t p = 0; p < k; p++) {
    const double* ap = a + p * DMR;
    const double* bp = b + p * DNR;
    for (int i = 0; i < DMR; i++)
      for (int j = 0; j < DNR; j++) acc[i][j] = fma(ap[i], bp[j], acc[i][j]);
  }
  const double al = *alpha, be = *beta;
  for (int i = 0; i < DMR; i++)
    for (int j = 0; j < DNR; j++) acc[i][j] = acc[i][j] * al;
  /* vucomisd sets ZF for equal and for unordered operands */
  if (be == 0.0 || isnan(be)) {
    for (int i = 0; i < DMR; i++)
      for (int j = 0; j < DNR; j++) c[i * rs_c + j * cs_c] = acc[i][j];
  } else {
    for (int i = 0; i < DMR; i++)
      for (int j = 0; j < DNR; j++) c[i * rs_c + j * cs_c] = fma(be, c[i * rs_c + j * cs_c], acc[i][j]);
  }
}

void oracle_ukr_s6x16(dim_t k, float* alpha, float* a, float* b, float* beta, float* c, inc_t rs_c, inc_t cs_c,
                      void* data, void* cntx) {
  (void)data;
  (void)cntx;
  float acc[SMR][SNR];
  for (int i = 0; i < SMR; i++)
    for (int j = 0; j < SNR; j++) acc[i][j] = 0.0f;
  for (dim_t p = 0; p < k; p++) {
    const float* ap = a + p * SMR;
    const float* bp = b + p * SNR;
    for (int i = 0; i < SMR; i++)
      for (int j = 0; j < SNR; j++) acc[i][j] = fmaf(ap[i], bp[j], acc[i][j]);
  }
  const float al = *alpha, be = *beta;
  for (int i = 0; i < SMR; i++)
    for (int j = 0; j < SNR; j++) acc[i][j] = acc[i][j] * al;
  if (be == 0.0f || isnan(be)) {
    for (int i = 0; i < SMR; i++)
      for (int j = 0; j < SNR; j++) c[i * rs_c + j * cs_c] = acc[i][j];
  } else {
    for (int i = 0; i < SMR; i++)
      for (int j = 0; j < SNR; j++) c[i * rs_c + j * cs_c] = fmaf(be, c[i * rs_c + j * cs_c], acc[i][j]);
  }
}

/* ------------------------------------------------------------------------ */
/* Thread team: the restatement of SpawnThreads + ThreadInfo::barrier.        */
/* ------------------------------------------------------------------------ */

typedef struct {
  pthread_mutex_t mu;
  pthread_cond_t cv;
  int count, nthreads;
  unsigned long generation;
} team_barrier_t;

static void team_barrier_init(team_barrier_t* b, int n) {
  pthread_mutex_init(&b->mu, NULL);
  pthread_cond_init(&b->cv, NULL);
  b->count = 0;
  b->nthreads = n;
  b->generation = 0;
}

static void team_barrier_wait(team_barrier_t* b) {
  if (b->nthreads == 1) return;
  pthread_mutex_lock(&b->mu);
  unsigned long gen = b->generation;
  if (++b->count == b->nthreads) {
    b->count = 0;
    b->generation++;
    pthread_cond_broadcast(&b->cv);
  } else {
    while (gen == b->generation) pthread_cond_wait(&b->cv, &b->mu);
  }
  pthread_mutex_unlock(&b->mu);
}

static void team_barrier_destroy(team_barrier_t* b) {
  pthread_mutex_destroy(&b->mu);
  pthread_cond_destroy(&b->cv);
}

/* ------------------------------------------------------------------------ */
/* The Goto loop nest, written once per element type through a macro.        */
/* ------------------------------------------------------------------------ */

#define GOTO_NC 3000
#define GOTO_KC 192
#define GOTO_MC 120

#define DEFINE_GOTO(T, SUF, MR, NR, UKR_T, DEFAULT_UKR)                                                          \
  typedef struct {                                                                                               \
    dim_t m, n, k;                                                                                               \
    T alpha, beta;                                                                                               \
    const T* A;                                                                                                  \
    inc_t rsa, csa;                                                                                              \
    const T* B;                                                                                                  \
    inc_t rsb, csb;                                                                                              \
    T* C;                                                                                                        \
    inc_t rsc, csc;                                                                                              \
    T* bpack; /* shared: ceil(NC/NR) panels of KC x NR */                                                        \
    T* apack; /* shared: ceil(MC/MR) panels of MR x KC */                                                        \
    UKR_T ukr;                                                                                                   \
    int nthreads;                                                                                                \
    team_barrier_t bar;                                                                                          \
  } goto_job_##SUF;                                                                                              \
                                                                                                                 \
  typedef struct {                                                                                               \
    goto_job_##SUF* job;                                                                                         \
    int tid;                                                                                                     \
  } goto_arg_##SUF;                                                                                              \
                                                                                                                 \
  static void* goto_worker_##SUF(void* p) {                                                                      \
    goto_arg_##SUF* arg = (goto_arg_##SUF*)p;                                                                    \
    goto_job_##SUF* J = arg->job;                                                                                \
    const int tid = arg->tid, nt = J->nthreads;                                                                  \
    T tmp[MR * NR];                                                                                              \
    T zero = (T)0;                                                                                               \
    for (dim_t jc = 0; jc < J->n; jc += GOTO_NC) {                                                               \
      const dim_t nc = (J->n - jc < GOTO_NC) ? J->n - jc : GOTO_NC;                                              \
      T beta_eff = J->beta; /* PartK: the first slab uses C's own scalar */                                      \
      for (dim_t pc = 0; pc < J->k; pc += GOTO_KC) {                                                             \
        const dim_t kc = (J->k - pc < GOTO_KC) ? J->k - pc : GOTO_KC;                                            \
        /* PackB: NR-wide column panels, element (y, i) of panel q at p[y*NR + i] */                             \
        const dim_t nbp = (nc + NR - 1) / NR;                                                                    \
        team_barrier_wait(&J->bar);                                                                              \
        for (dim_t q = tid; q < nbp; q += nt) {                                                                  \
          T* pp = J->bpack + q * (GOTO_KC * NR);                                                                 \
          for (dim_t y = 0; y < kc; y++)                                                                         \
            for (dim_t i = 0; i < NR; i++) {                                                                     \
              dim_t x = q * NR + i;                                                                              \
              pp[y * NR + i] = (x < nc) ? J->B[(pc + y) * J->rsb + (jc + x) * J->csb] : zero;                    \
            }                                                                                                    \
        }                                                                                                        \
        team_barrier_wait(&J->bar);                                                                              \
        for (dim_t ic = 0; ic < J->m; ic += GOTO_MC) {                                                           \
          const dim_t mc = (J->m - ic < GOTO_MC) ? J->m - ic : GOTO_MC;                                          \
          const dim_t nap = (mc + MR - 1) / MR;                                                                  \
          /* PackA: MR-tall row panels, element (i, x) of panel q at p[x*MR + i] */                              \
          team_barrier_wait(&J->bar);                                                                            \
          for (dim_t q = tid; q < nap; q += nt) {                                                                \
            T* pp = J->apack + q * (GOTO_KC * MR);                                                               \
            for (dim_t x = 0; x < kc; x++)                                                                       \
              for (dim_t i = 0; i < MR; i++) {                                                                   \
                dim_t y = q * MR + i;                                                                            \
                pp[x * MR + i] = (y < mc) ? J->A[(ic + y) * J->rsa + (pc + x) * J->csa] : zero;                  \
              }                                                                                                  \
          }                                                                                                      \
          team_barrier_wait(&J->bar);                                                                            \
          /* ParallelN<NR, TheRest>: contiguous range of NR panels per thread */                                 \
          const dim_t per = (nbp - 1) / nt + 1;                                                                  \
          const dim_t q0 = per * tid;                                                                            \
          const dim_t q1 = (q0 + per < nbp) ? q0 + per : nbp;                                                    \
          for (dim_t q = q0; q < q1; q++) {                                                                      \
            const dim_t jr = q * NR;                                                                             \
            const dim_t ln = (nc - jr < NR) ? nc - jr : NR;                                                      \
            T* bp = J->bpack + q * (GOTO_KC * NR);                                                               \
            for (dim_t r = 0; r < nap; r++) {                                                                    \
              const dim_t ir = r * MR;                                                                           \
              const dim_t lm = (mc - ir < MR) ? mc - ir : MR;                                                    \
              T* ap = J->apack + r * (GOTO_KC * MR);                                                             \
              T* cp = J->C + (ic + ir) * J->rsc + (jc + jr) * J->csc;                                            \
              T al = J->alpha;                                                                                   \
              if (lm == MR && ln == NR) {                                                                        \
                T be = beta_eff;                                                                                 \
                J->ukr(kc, &al, ap, bp, &be, cp, J->rsc, J->csc, NULL, NULL);                                    \
              } else {                                                                                           \
                /* kernel_nm.rs:77-95: tmp (column-major MR x NR) with beta 0 */                                 \
                T tz = zero;                                                                                     \
                J->ukr(kc, &al, ap, bp, &tz, tmp, 1, MR, NULL, NULL);                                            \
                for (dim_t ii = 0; ii < lm; ii++)                                                                \
                  for (dim_t jj = 0; jj < ln; jj++) {                                                            \
                    T tau = tmp[ii + jj * MR];                                                                   \
                    T* cij = cp + ii * J->rsc + jj * J->csc;                                                     \
                    T prod = beta_eff * (*cij);                                                                  \
                    *cij = tau + prod;                                                                           \
                  }                                                                                              \
              }                                                                                                  \
            }                                                                                                    \
          }                                                                                                      \
        }                                                                                                        \
        beta_eff = (T)1; /* part.rs:105 */                                                                       \
      }                                                                                                          \
    }                                                                                                            \
    return NULL;                                                                                                 \
  }                                                                                                              \
                                                                                                                 \
  int oracle_goto_##SUF##gemm(dim_t m, dim_t n, dim_t k, T alpha, const T* A, inc_t rsa, inc_t csa, const T* B,  \
                              inc_t rsb, inc_t csb, T beta, T* C, inc_t rsc, inc_t csc, int nthreads, void* ukr) { \
    if (m < 0 || n < 0 || k < 0) return -1;                                                                      \
    if (m == 0 || n == 0) return 0;                                                                              \
    if (nthreads < 1) nthreads = 1;                                                                              \
    goto_job_##SUF J;                                                                                            \
    memset(&J, 0, sizeof(J));                                                                                    \
    J.m = m; J.n = n; J.k = k; J.alpha = alpha; J.beta = beta;                                                   \
    J.A = A; J.rsa = rsa; J.csa = csa; J.B = B; J.rsb = rsb; J.csb = csb;                                        \
    J.C = C; J.rsc = rsc; J.csc = csc;                                                                           \
    J.ukr = ukr ? (UKR_T)ukr : DEFAULT_UKR;                                                                      \
    J.nthreads = nthreads;                                                                                       \
    size_t nb = (size_t)((GOTO_NC + NR - 1) / NR) * GOTO_KC * NR;                                                \
    size_t na = (size_t)((GOTO_MC + MR - 1) / MR) * GOTO_KC * MR;                                                \
    J.bpack = (T*)aligned_alloc(4096, ((nb * sizeof(T) + 4095) / 4096) * 4096);                                  \
    J.apack = (T*)aligned_alloc(4096, ((na * sizeof(T) + 4095) / 4096) * 4096);                                  \
    if (!J.bpack || !J.apack) { free(J.bpack); free(J.apack); return -2; }                                       \
    if (k == 0) {                                                                                                \
      /* no k slab runs, so the reference leaves C untouched */                                                  \
      free(J.bpack); free(J.apack); return 0;                                                                    \
    }                                                                                                            \
    team_barrier_init(&J.bar, nthreads);                                                                         \
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nthreads);                                            \
    goto_arg_##SUF* args = (goto_arg_##SUF*)malloc(sizeof(goto_arg_##SUF) * nthreads);                           \
    for (int t = 0; t < nthreads; t++) { args[t].job = &J; args[t].tid = t; }                                    \
    for (int t = 1; t < nthreads; t++) pthread_create(&th[t], NULL, goto_worker_##SUF, &args[t]);                \
    goto_worker_##SUF(&args[0]);                                                                                 \
    for (int t = 1; t < nthreads; t++) pthread_join(th[t], NULL);                                                \
    team_barrier_destroy(&J.bar);                                                                                \
    free(th); free(args); free(J.bpack); free(J.apack);                                                          \
    return 0;                                                                                                    \
  }

DEFINE_GOTO(double, d, DMR, DNR, dukr_t, oracle_ukr_d6x8)
DEFINE_GOTO(float, s, SMR, SNR, sukr_t, oracle_ukr_s6x16)

/* ------------------------------------------------------------------------ */
/* Double-double accumulated GEMM: the high-accuracy oracle.                 */
/* ------------------------------------------------------------------------ */

/* error-free transformations (Knuth TwoSum, fma-based TwoProd) */
static inline void two_sum(double a, double b, double* s, double* e) {
  double x = a + b;
  double bv = x - a;
  double av = x - bv;
  *s = x;
  *e = (a - av) + (b - bv);
}

static inline void dd_add_d(double* hi, double* lo, double p, double pe) {
  /* (hi, lo) += (p, pe) */
  double s, e;
  two_sum(*hi, p, &s, &e);
  e += *lo + pe;
  double s2 = s + e;
  *lo = e - (s2 - s);
  *hi = s2;
}

typedef struct {
  dim_t m, n, k;
  double alpha, beta;
  const double *A, *B, *C0;
  inc_t rsa, csa, rsb, csb, rsc, csc;
  double *Cout, *Mag;
  inc_t rso, cso;
  const int64_t *ii, *jj; /* optional entry list */
  int64_t count;
  int nthreads;
  int tid;
} dd_job;

static void dd_entry(const dd_job* J, dim_t i, dim_t j, double* out, double* mag) {
  double hi = 0.0, lo = 0.0, absum = 0.0;
  for (dim_t p = 0; p < J->k; p++) {
    double a = J->A[i * J->rsa + p * J->csa];
    double b = J->B[p * J->rsb + j * J->csb];
    double pr = a * b;
    double pe = fma(a, b, -pr);
    dd_add_d(&hi, &lo, pr, pe);
    absum += fabs(pr);
  }
  /* alpha * (hi + lo) in double-double */
  double ph = J->alpha * hi;
  double pl = fma(J->alpha, hi, -ph) + J->alpha * lo;
  double rh = ph, rl = pl;
  double cmag = 0.0;
  if (J->C0 && J->beta != 0.0) {
    double c = J->C0[i * J->rsc + j * J->csc];
    double q = J->beta * c;
    double qe = fma(J->beta, c, -q);
    dd_add_d(&rh, &rl, q, qe);
    cmag = fabs(q);
  }
  *out = rh + rl;
  if (mag) *mag = fabs(J->alpha) * absum + cmag;
}

static void* dd_worker(void* p) {
  dd_job* J = (dd_job*)p;
  if (J->ii) {
    for (int64_t e = J->tid; e < J->count; e += J->nthreads) {
      double o, mg;
      dd_entry(J, J->ii[e], J->jj[e], &o, &mg);
      J->Cout[e] = o;
      if (J->Mag) J->Mag[e] = mg;
    }
  } else {
    for (dim_t j = J->tid; j < J->n; j += J->nthreads)
      for (dim_t i = 0; i < J->m; i++) {
        double o, mg;
        dd_entry(J, i, j, &o, &mg);
        J->Cout[i * J->rso + j * J->cso] = o;
        if (J->Mag) J->Mag[i * J->rso + j * J->cso] = mg;
      }
  }
  return NULL;
}

static int run_dd(dd_job* base) {
  int nt = base->nthreads < 1 ? 1 : base->nthreads;
  dd_job* jobs = (dd_job*)malloc(sizeof(dd_job) * nt);
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * nt);
  for (int t = 0; t < nt; t++) {
    jobs[t] = *base;
    jobs[t].nthreads = nt;
    jobs[t].tid = t;
  }
  for (int t = 1; t < nt; t++) pthread_create(&th[t], NULL, dd_worker, &jobs[t]);
  dd_worker(&jobs[0]);
  for (int t = 1; t < nt; t++) pthread_join(th[t], NULL);
  free(jobs);
  free(th);
  return 0;
}

/* Cout (m x n, strides rso/cso) = beta*C0 + alpha*A*B accumulated in
 * double-double and rounded once; Mag (optional) = |alpha||A||B| + |beta||C0|.
 * C0 may be NULL (treated as zero). */
int oracle_dd_dgemm(dim_t m, dim_t n, dim_t k, double alpha, const double* A, inc_t rsa, inc_t csa, const double* B,
                    inc_t rsb, inc_t csb, double beta, const double* C0, inc_t rsc, inc_t csc, double* Cout, double* Mag,
                    inc_t rso, inc_t cso, int nthreads) {
  dd_job J;
  memset(&J, 0, sizeof(J));
  J.m = m; J.n = n; J.k = k; J.alpha = alpha; J.beta = beta;
  J.A = A; J.rsa = rsa; J.csa = csa; J.B = B; J.rsb = rsb; J.csb = csb;
  J.C0 = C0; J.rsc = rsc; J.csc = csc; J.Cout = Cout; J.Mag = Mag; J.rso = rso; J.cso = cso;
  J.nthreads = nthreads;
  return run_dd(&J);
}

/* Same as oracle_dd_dgemm for a list of (ii[e], jj[e]) entries only; writes
 * Cout[e] and Mag[e]. Used to check full-size results on a sample. */
int oracle_dd_dgemm_entries(dim_t m, dim_t n, dim_t k, double alpha, const double* A, inc_t rsa, inc_t csa,
                            const double* B, inc_t rsb, inc_t csb, double beta, const double* C0, inc_t rsc, inc_t csc,
                            const int64_t* ii, const int64_t* jj, int64_t count, double* Cout, double* Mag,
                            int nthreads) {
  dd_job J;
  memset(&J, 0, sizeof(J));
  J.m = m; J.n = n; J.k = k; J.alpha = alpha; J.beta = beta;
  J.A = A; J.rsa = rsa; J.csa = csa; J.B = B; J.rsb = rsb; J.csb = csb;
  J.C0 = C0; J.rsc = rsc; J.csc = csc; J.Cout = Cout; J.Mag = Mag;
  J.ii = ii; J.jj = jj; J.count = count;
  J.nthreads = nthreads;
  return run_dd(&J);
}

/* ------------------------------------------------------------------------ */
/* The reference's randomized check (src/util.rs:55-85):                      */
/*   ||C w - A (B w)||_F^2 for a caller-supplied vector w (the reference      */
/*   draws w from an unseeded RNG; here the caller seeds it).                 */
/* ------------------------------------------------------------------------ */

double oracle_freivalds_d(dim_t m, dim_t n, dim_t k, const double* A, inc_t rsa, inc_t csa, const double* B,
                          inc_t rsb, inc_t csb, const double* C, inc_t rsc, inc_t csc, const double* w) {
  double* bw = (double*)calloc((size_t)(k > 0 ? k : 1), sizeof(double));
  double res = 0.0;
  for (dim_t p = 0; p < k; p++) {
    double s = 0.0;
    for (dim_t j = 0; j < n; j++) s += B[p * rsb + j * csb] * w[j];
    bw[p] = s;
  }
  for (dim_t i = 0; i < m; i++) {
    double abw = 0.0, cw = 0.0;
    for (dim_t p = 0; p < k; p++) abw += A[i * rsa + p * csa] * bw[p];
    for (dim_t j = 0; j < n; j++) cw += C[i * rsc + j * csc] * w[j];
    double d = cw - abw;
    res += d * d;
  }
  free(bw);
  return res;
}

/*
 * pmmc_oracle.c -- plain-C restatement of the reference's CPU annealers.
 *
 * TEST INFRASTRUCTURE ONLY (see pmmc_oracle.h): the checker for the CUDA
 * path, never part of it.  Each function names the reference file:line it
 * restates.  Types follow the reference expression by expression: vector3 is
 * three floats (src/thirdparty/mtxlib.h:84-123) whose length() is a float
 * (mtxlib.cpp:322), scores accumulate in double, and a float-typed
 * subexpression such as `(v.length() - e) / e` stays float before it is
 * widened.  Compile with -ffp-contract=off.
 */
#include "pmmc_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------ */
/* vector3 helpers (mtxlib.cpp:322-345, common.cpp:39-46)             */
/* ------------------------------------------------------------------ */
static float v_len(float x, float y, float z) {
  float s = x * x + y * y;
  s = s + z * z;
  return (float)sqrt((double)s);
}

/* angle(v1, v2) = 1 - (dot(n1, n2) + 1) / 2 with both vectors normalised. */
static float v_angle(const float a[3], const float b[3]) {
  float ma = v_len(a[0], a[1], a[2]);
  ma = ma > 0.0f ? 1.0f / ma : 0.0f;
  float mb = v_len(b[0], b[1], b[2]);
  mb = mb > 0.0f ? 1.0f / mb : 0.0f;
  float ax = a[0] * ma, ay = a[1] * ma, az = a[2] * ma;
  float bx = b[0] * mb, by = b[1] * mb, bz = b[2] * mb;
  float dot = ax * bx + ay * by;
  dot = dot + az * bz;
  return 1.0f - (dot + 1.0f) / 2.0f;
}

/* SphericalContainer::boundaryPenalty (src/include/SphericalContainer.hpp:
 * 109-122), centre at the origin. */
static float sphere_pen(const float *p, float radius) {
  float ds = p[0] * p[0] + p[1] * p[1];
  ds = ds + p[2] * p[2];
  float rs = radius * radius;
  if (ds <= rs)
    return 0.0f;
  float d = sqrtf(ds);
  float o = d - radius;
  return o * o;
}

/* ------------------------------------------------------------------ */
/* Philox4x32-10 (J. Salmon, M. Moraes, R. Dror, D. Shaw, "Parallel    */
/* random numbers: as easy as 1, 2, 3", SC'11).                        */
/* ------------------------------------------------------------------ */
#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                       uint32_t out[4]) {
  uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
  uint32_t k0 = key[0], k1 = key[1];
  for (int r = 0; r < 10; ++r) {
    uint64_t p0 = (uint64_t)PHILOX_M0 * c0;
    uint64_t p1 = (uint64_t)PHILOX_M1 * c2;
    uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
    uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
    c0 = hi1 ^ c1 ^ k0;
    c1 = lo1;
    c2 = hi0 ^ c3 ^ k1;
    c3 = lo0;
    k0 += PHILOX_W0;
    k1 += PHILOX_W1;
  }
  out[0] = c0;
  out[1] = c1;
  out[2] = c2;
  out[3] = c3;
}

float orc_u01(uint32_t x) { return (float)(x >> 8) * (1.0f / 16777216.0f); }

/* ------------------------------------------------------------------ */
/* Random-number source                                                */
/* ------------------------------------------------------------------ */
typedef struct {
  orc_rng *r;
  const int *movable; /* philox: indices of non-fixed beads */
  int n_movable;
  float disp_u[3];    /* philox: cached displacement draws of the move */
  int u_from_bead;    /* philox, smoothing: the Metropolis uniform is the
                         bead draw's fractional part (one block a move) */
  float bead_u;
} rng_ctx;

/* libc draws, common.cpp:10-18: random(range) = rand() % range,
 * random_uniform() = rand() / (float)RAND_MAX. */
static float libc_uniform(void) { return (float)rand() / (float)RAND_MAX; }

static void philox_block(const orc_rng *r, uint32_t tag, uint32_t out[4]) {
  uint32_t ctr[4] = {(uint32_t)r->move, (uint32_t)(r->move >> 32), r->chain,
                     tag};
  uint32_t key[2] = {(uint32_t)r->seed, (uint32_t)(r->seed >> 32)};
  orc_philox4x32_10(ctr, key, out);
}

/* Bead draw.  libc: rand() % size (the caller skips fixed beads as the
 * reference does).  philox: one of the movable beads, uniformly. */
static int draw_bead(rng_ctx *c, int size) {
  if (c->r->kind == ORC_RNG_LIBC)
    return rand() % size;
  uint32_t o[4];
  philox_block(c->r, 0u, o);
  c->disp_u[0] = orc_u01(o[1]);
  c->disp_u[1] = orc_u01(o[2]);
  c->disp_u[2] = orc_u01(o[3]);
  const uint64_t prod = (uint64_t)o[0] * (uint32_t)c->n_movable;
  uint32_t k = (uint32_t)(prod >> 32);
  /* the low word: the draw's fractional part within bead k's interval */
  c->bead_u = orc_u01((uint32_t)prod);
  return c->movable[k];
}

/* random_vector(max, in2D) (common.cpp:20-25).  GCC evaluates the vector3
 * constructor's arguments right to left, so the first libc draw is z. */
static void draw_disp(rng_ctx *c, float max, int in2d, float d[3]) {
  if (c->r->kind == ORC_RNG_LIBC) {
    if (in2d) {
      d[2] = 0.0f;
      d[1] = (2.0f * libc_uniform() - 1.0f) * max;
      d[0] = (2.0f * libc_uniform() - 1.0f) * max;
    } else {
      d[2] = (2.0f * libc_uniform() - 1.0f) * max;
      d[1] = (2.0f * libc_uniform() - 1.0f) * max;
      d[0] = (2.0f * libc_uniform() - 1.0f) * max;
    }
    return;
  }
  d[0] = (2.0f * c->disp_u[0] - 1.0f) * max;
  d[1] = (2.0f * c->disp_u[1] - 1.0f) * max;
  d[2] = in2d ? 0.0f : (2.0f * c->disp_u[2] - 1.0f) * max;
}

/* withChance(chance) = random_uniform() < chance (common.cpp:326). */
static int draw_chance(rng_ctx *c, float chance) {
  if (c->r->kind == ORC_RNG_LIBC)
    return libc_uniform() < chance;
  if (c->u_from_bead)
    return c->bead_u < chance;
  uint32_t o[4];
  philox_block(c->r, 1u, o);
  return orc_u01(o[0]) < chance;
}

static void end_move(rng_ctx *c) {
  if (c->r->kind == ORC_RNG_PHILOX)
    c->r->move++;
}

static int *movable_list(int n, const unsigned char *fixed, int *cnt) {
  int *m = (int *)malloc(sizeof(int) * (n > 0 ? n : 1));
  int k = 0;
  for (int i = 0; i < n; ++i)
    if (!fixed || !fixed[i])
      m[k++] = i;
  *cnt = k;
  return m;
}

static void rng_begin(rng_ctx *c, orc_rng *r, int n,
                      const unsigned char *fixed) {
  c->r = r;
  c->movable = NULL;
  c->n_movable = 0;
  c->u_from_bead = 0;
  c->bead_u = 0.0f;
  if (r->kind == ORC_RNG_LIBC) {
    srand((unsigned)r->seed);
  } else {
    c->movable = movable_list(n, fixed, &c->n_movable);
  }
}

static void rng_end(rng_ctx *c) { free((void *)c->movable); }

/* ------------------------------------------------------------------ */
/* Loop constraints: rebuildActiveLoopMap (LooperSolver.hpp:3318-3337)  */
/* keys (min,max) in std::map order, the last constraint of a key wins. */
/* ------------------------------------------------------------------ */
typedef struct {
  int a, b;
  float k, r0;
} loop_ent;

static int loop_cmp(const void *x, const void *y) {
  const loop_ent *p = (const loop_ent *)x, *q = (const loop_ent *)y;
  if (p->a != q->a)
    return p->a < q->a ? -1 : 1;
  if (p->b != q->b)
    return p->b < q->b ? -1 : 1;
  return 0;
}

static loop_ent *build_loops(int n, int n_loops, const int *li, const int *lj,
                             const float *lk, const float *lr0, int *cnt) {
  loop_ent *e = (loop_ent *)malloc(sizeof(loop_ent) * (n_loops > 0 ? n_loops : 1));
  int m = 0;
  for (int c = 0; c < n_loops; ++c) {
    int i = li[c], j = lj[c];
    if (i < 0 || i >= n || j < 0 || j >= n)
      continue;
    loop_ent x;
    x.a = i < j ? i : j;
    x.b = i < j ? j : i;
    x.k = lk[c];
    x.r0 = lr0[c];
    int found = -1;
    for (int t = 0; t < m; ++t)
      if (e[t].a == x.a && e[t].b == x.b)
        found = t;
    if (found >= 0)
      e[found] = x; /* active_loop_map[key] = c : the later one wins */
    else
      e[m++] = x;
  }
  qsort(e, m, sizeof(loop_ent), loop_cmp);
  *cnt = m;
  return e;
}

static double loop_energy(const float *pos, const loop_ent *e, int m,
                          int moved) {
  double sc = 0.0;
  for (int t = 0; t < m; ++t) {
    if (moved >= 0 && e[t].a != moved && e[t].b != moved)
      continue;
    const float *pa = pos + 3 * e[t].a, *pb = pos + 3 * e[t].b;
    double d = v_len(pa[0] - pb[0], pa[1] - pb[1], pa[2] - pb[2]);
    double delta = d - e[t].r0;
    sc += e[t].k * delta * delta;
  }
  return sc;
}

/* ------------------------------------------------------------------ */
/* Arc level                                                           */
/* ------------------------------------------------------------------ */
/* calcScoreDistancesActiveRegion() (LooperSolver.hpp:3215-3246). */
static double arcs_dist_full(int n, const float *pos, const float *ed,
                             const orc_params *p, int with_springs,
                             int with_repulsion) {
  double sc = 0.0;
  for (int i = 0; i < n; ++i) {
    for (int j = i + 1; j < n; ++j) {
      const float *a = pos + 3 * i, *b = pos + 3 * j;
      float len = v_len(a[0] - b[0], a[1] - b[1], a[2] - b[2]);
      float e = ed[(size_t)i * n + j];
      if (e < 0.0f) {
        if (with_repulsion)
          sc += 1.0f / len;
        continue;
      }
      if (e < 1e-6)
        continue;
      if (!with_springs)
        continue;
      float t = (len - e) / e;
      double diff = t;
      sc += diff * diff * (diff >= 0.0f ? p->k_stretch : p->k_squeeze);
    }
  }
  return sc;
}

/* calcScoreDistancesActiveRegion(int) (LooperSolver.hpp:3250-3281). */
static double arcs_dist_local(int n, const float *pos, const float *ed,
                              const orc_params *p, int moved) {
  double sc = 0.0;
  const float *m = pos + 3 * moved;
  for (int i = 0; i < n; ++i) {
    if (i == moved)
      continue;
    const float *b = pos + 3 * i;
    float e = ed[(size_t)i * n + moved];
    if (e < 0.0f)
      continue;
    if (e < 1e-6)
      continue;
    float len = v_len(m[0] - b[0], m[1] - b[1], m[2] - b[2]);
    float t = (len - e) / e;
    double diff = t;
    sc += diff * diff * (diff >= 0.0f ? p->k_stretch : p->k_squeeze);
  }
  return sc;
}

double orc_arcs_full_score(int n, const float *pos, const float *exp_dist,
                           int n_loops, const int *loop_i, const int *loop_j,
                           const float *loop_k, const float *loop_r0,
                           const orc_params *p) {
  int m;
  loop_ent *e = build_loops(n, n_loops, loop_i, loop_j, loop_k, loop_r0, &m);
  double sc = arcs_dist_full(n, pos, exp_dist, p, 1, 1) + loop_energy(pos, e, m, -1);
  if (p->sphere_radius > 0.0f)
    for (int k = 0; k < n; ++k)
      sc += sphere_pen(pos + 3 * k, p->sphere_radius);
  free(e);
  return sc;
}

double orc_arcs_spring_score(int n, const float *pos, const float *exp_dist,
                             int n_loops, const int *loop_i, const int *loop_j,
                             const float *loop_k, const float *loop_r0,
                             const orc_params *p) {
  int m;
  loop_ent *e = build_loops(n, n_loops, loop_i, loop_j, loop_k, loop_r0, &m);
  double sc = arcs_dist_full(n, pos, exp_dist, p, 1, 0) + loop_energy(pos, e, m, -1);
  if (p->sphere_radius > 0.0f)
    for (int k = 0; k < n; ++k)
      sc += sphere_pen(pos + 3 * k, p->sphere_radius);
  free(e);
  return sc;
}

double orc_arcs_repulsion(int n, const float *pos, const float *exp_dist) {
  orc_params p;
  memset(&p, 0, sizeof(p));
  return arcs_dist_full(n, pos, exp_dist, &p, 0, 1);
}

double orc_arcs_local_score(int n, const float *pos, const float *exp_dist,
                            int n_loops, const int *loop_i, const int *loop_j,
                            const float *loop_k, const float *loop_r0,
                            const orc_params *p, int moved) {
  int m;
  loop_ent *e = build_loops(n, n_loops, loop_i, loop_j, loop_k, loop_r0, &m);
  double sc = arcs_dist_local(n, pos, exp_dist, p, moved) + loop_energy(pos, e, m, moved);
  if (p->sphere_radius > 0.0f)
    sc += sphere_pen(pos + 3 * moved, p->sphere_radius);
  free(e);
  return sc;
}

/* LooperSolver::MonteCarloArcs (LooperSolver.hpp:4670-4796).  Differences
 * only where the reference has no counterpart: the Philox source picks among
 * movable beads directly and keeps the pre-move position on rejection (as the
 * CUDA kernels do) instead of subtracting the displacement back.
 *
 * ORC_SCHEDULE_GPU restates the schedule of the reference's arc kernel
 * (MonteCarloArcsKernel, src/ParallelMonteCarloArcs.cu:494-655) around the
 * same moves: blocks of 256 moves while fewer than milestone_steps moves are
 * done (:522,631), so the cap is milestone_steps rounded up to 256 and no
 * move at all when it is <= 0; an uphill move is tested only when T > 0 and
 * the previous score is > 0 (:598-603), otherwise it is rejected without a
 * draw; after every block the milestone predicate (:635-641) -- the CPU one
 * with the ratio test guarded by milestone_score > 1e-10 -- counts
 * consecutive misses (:643-646), and the chain stops when they reach
 * milestone_fails or the score drops below 1e-5 (:648-650).  The kernel keeps
 * its score in float; this restatement keeps it in double, the precision
 * form the GPU path reproduces. */
static double ext_full(int n, const float *pos, const orc_ext *x);
static double ext_local(int n, const float *pos, const orc_ext *x, int moved);

void orc_arcs_anneal(int n, float *pos, const unsigned char *fixed,
                     const float *exp_dist, int n_loops, const int *loop_i,
                     const int *loop_j, const float *loop_k,
                     const float *loop_r0, const orc_params *p,
                     float step_size, orc_rng *rng, orc_result *res) {
  orc_arcs_anneal_ext(n, pos, fixed, exp_dist, n_loops, loop_i, loop_j, loop_k, loop_r0, p,
                      NULL, step_size, rng, res);
}

void orc_arcs_anneal_ext(int n, float *pos, const unsigned char *fixed,
                         const float *exp_dist, int n_loops, const int *loop_i,
                         const int *loop_j, const float *loop_k,
                         const float *loop_r0, const orc_params *p,
                         const orc_ext *x, float step_size, orc_rng *rng,
                         orc_result *res) {
  int m;
  loop_ent *e = build_loops(n, n_loops, loop_i, loop_j, loop_k, loop_r0, &m);
  rng_ctx c;
  rng_begin(&c, rng, n, fixed);
  memset(res, 0, sizeof(*res));

  double T = p->max_temp, dt = p->dt_temp, tp;
  double score_curr = arcs_dist_full(n, pos, exp_dist, p, 1, 1) + loop_energy(pos, e, m, -1);
  if (p->sphere_radius > 0.0f)
    for (int k = 0; k < n; ++k)
      score_curr += sphere_pen(pos + 3 * k, p->sphere_radius);
  if (x)
    score_curr += ext_full(n, pos, x);
  double score_prev = score_curr, milestone_score = score_curr;
  int64_t success = 0, milestone_success = 0, i = 1;
  int philox = rng->kind == ORC_RNG_PHILOX;
  int gpu = p->schedule == ORC_SCHEDULE_GPU;
  int64_t cap = p->milestone_steps > 0 ? ((int64_t)p->milestone_steps + 255) / 256 * 256 : 0;
  int misses = 0;

  res->best = score_curr;
  if ((philox && c.n_movable == 0) || (gpu && cap == 0)) { /* nothing moves */
    res->score = score_curr;
    goto done;
  }
  for (;;) {
    int pb = draw_bead(&c, n);
    res->proposals++;
    if (fixed && fixed[pb]) {
      /* the reference stops the program here (error(), :4718-4719) */
      fprintf(stderr, "oracle: cluster fixed during arcs\n");
      res->score = score_curr;
      res->moves = -1;
      goto done;
    }
    float *q = pos + 3 * pb;
    double lp = arcs_dist_local(n, pos, exp_dist, p, pb) + loop_energy(pos, e, m, pb);
    if (p->sphere_radius > 0.0f)
      lp += sphere_pen(q, p->sphere_radius);
    if (x)
      lp += ext_local(n, pos, x, pb);
    float d[3], old[3] = {q[0], q[1], q[2]};
    draw_disp(&c, step_size, p->use2d, d);
    q[0] += d[0];
    q[1] += d[1];
    q[2] += d[2];
    double lc = arcs_dist_local(n, pos, exp_dist, p, pb) + loop_energy(pos, e, m, pb);
    if (p->sphere_radius > 0.0f)
      lc += sphere_pen(q, p->sphere_radius);
    if (x)
      lc += ext_local(n, pos, x, pb);
    score_curr = score_curr - lp + lc;
    int ok = score_curr <= score_prev;
    if (!ok && (!gpu || (T > 0.0 && score_prev > 0.0))) {
      tp = p->jump_scale * exp(-p->jump_coef * (score_curr / score_prev) / T);
      ok = draw_chance(&c, (float)tp);
    }
    if (ok) {
      success++;
      milestone_success++;
      if (score_curr < res->best) res->best = score_curr;
    } else {
      if (philox) {
        q[0] = old[0];
        q[1] = old[1];
        q[2] = old[2];
      } else {
        q[0] -= d[0];
        q[1] -= d[1];
        q[2] -= d[2];
      }
      score_curr = score_prev;
    }
    end_move(&c);
    T *= dt;
    if (gpu) {
      if (i % 256 == 0) {
        int miss = (score_curr > p->improvement * milestone_score &&
                    milestone_success < p->min_successes) ||
                   score_curr < 1e-5 ||
                   (milestone_score > 1e-10 && score_curr / milestone_score > 0.9999);
        misses = miss ? misses + 1 : 0;
        if (misses >= p->milestone_fails || score_curr < 1e-5)
          break;
        milestone_score = score_curr;
        milestone_success = 0;
        if (i >= cap)
          break;
      }
    } else if (i % p->milestone_steps == 0) {
      if ((score_curr > p->improvement * milestone_score &&
           milestone_success < p->min_successes) ||
          score_curr < 1e-5 || score_curr / milestone_score > 0.9999)
        break;
      milestone_score = score_curr;
      milestone_success = 0;
    }
    if (p->max_moves > 0 && i >= p->max_moves)
      break;
    score_prev = score_curr;
    i++;
  }
  res->score = score_curr;
  res->moves = i;
  res->accepted = success;
done:
  rng_end(&c);
  free(e);
}

/* ------------------------------------------------------------------ */
/* Expected-distance heatmap (createDistanceHeatmap)                   */
/* ------------------------------------------------------------------ */
void orc_distance_heatmap(int n, const float *contact, int diag, float scale,
                          float power, float stretching, float *dist,
                          float *avg_out, float *max_out) {
  for (int i = 0; i < n; ++i)
    for (int j = i; j < n; ++j) {
      const float val = contact[(size_t)i * n + j];
      float d;
      if ((double)val < 1e-6)
        d = 0.0f;
      else
        d = abs(i - j) < diag ? -1.0f : scale * powf(val, power);
      dist[(size_t)i * n + j] = d;
      dist[(size_t)j * n + i] = d;
    }
  /* Heatmap::getDiagonalSize: the first offset with a value above 1e-6 */
  int w = 0, found = 0;
  for (int k = 0; k < n && !found; ++k)
    for (int i = 0; i + k < n; ++i)
      if (dist[(size_t)i * n + i + k] > 1e-6) {
        w = k;
        found = 1;
        break;
      }
  /* Heatmap::getAvg: float running sum in row order */
  float ret = 0.0f;
  int cnt = 0;
  for (int i = 0; i < n; ++i)
    for (int j = i + w; j < n; ++j) {
      ret += dist[(size_t)i * n + j];
      cnt++;
    }
  const float avg = ret / cnt;
  const float max_dist = avg * stretching;
  for (size_t k = 0; k < (size_t)n * n; ++k)
    if (dist[k] > max_dist) dist[k] = max_dist;
  *avg_out = avg;
  *max_out = max_dist;
}

/* ------------------------------------------------------------------ */
/* Equidistant model (gpuHelper's CPU path)                            */
/* ------------------------------------------------------------------ */
long long orc_equidistant(int n, const int *gpos, const float *pos, int first_end,
                          int last_start, int pos_start, int pos_stop, int res,
                          float *out, long long cap) {
  const long long out_size = (long long)((pos_stop - pos_start + 1) / res + 1);
  for (long long idx = 0; idx < out_size && idx < cap; ++idx) {
    const long long p = pos_start + (long long)res * idx;
    float *o = out + 3 * idx;
    if (p < first_end) {
      memcpy(o, pos, 3 * sizeof(float));
      continue;
    }
    if (p >= last_start) {
      memcpy(o, pos + 3 * (n - 1), 3 * sizeof(float));
      continue;
    }
    int prev = -1, found = 0;
    for (int i = 0; i < n; ++i) {
      if (p < gpos[i] && prev >= 0) {
        const float *p1 = pos + 3 * prev, *p2 = pos + 3 * i;
        float p0[3], p3[3];
        for (int c = 0; c < 3; ++c) {
          p0[c] = i > 1 ? pos[3 * (i - 2) + c] : 2.0f * p1[c] - p2[c];
          p3[c] = i + 1 < n ? pos[3 * (i + 1) + c] : 2.0f * p2[c] - p1[c];
        }
        const float t = (float)(p - gpos[prev]) / (float)(gpos[i] - gpos[prev]);
        const float t2 = t * t, t3 = t2 * t;
        const float b1 = 0.5f * (-t3 + 2.0f * t2 - t);
        const float b2 = 0.5f * (3.0f * t3 - 5.0f * t2 + 2.0f);
        const float b3 = 0.5f * (-3.0f * t3 + 4.0f * t2 + t);
        const float b4 = 0.5f * (t3 - t2);
        for (int c = 0; c < 3; ++c) o[c] = p0[c] * b1 + p1[c] * b2 + p2[c] * b3 + p3[c] * b4;
        found = 1;
        break;
      }
      prev = i;
    }
    if (!found && prev >= 0) memcpy(o, pos + 3 * prev, 3 * sizeof(float));
  }
  return out_size;
}

/* ------------------------------------------------------------------ */
/* Heatmap level                                                       */
/* ------------------------------------------------------------------ */
/* getChromosomeHeatmapBoundary (LooperSolver.hpp:6034-6050). */
static void hm_bounds(int n_bounds, const int *b, int p, int *st, int *en) {
  if (n_bounds == 0)
    return;
  if (p < 0 || p > b[n_bounds - 1])
    return;
  for (int i = 0; i + 1 < n_bounds; ++i)
    if (b[i] <= p && p < b[i + 1]) {
      *st = b[i];
      *en = b[i + 1] - 1;
      return;
    }
}

static double hm_local(int n, const float *pos, const float *h, int diag,
                       int n_bounds, const int *bounds, int moved) {
  double err = 0.0;
  int st = 0, en = n - 1;
  if (n_bounds > 0)
    hm_bounds(n_bounds, bounds, moved, &st, &en);
  const float *m = pos + 3 * moved;
  for (int i = st; i <= en; ++i) {
    if (abs(i - moved) >= diag) {
      float hv = h[(size_t)i * n + moved];
      if (hv < 1e-6)
        continue;
      const float *b = pos + 3 * i;
      float d = v_len(b[0] - m[0], b[1] - m[1], b[2] - m[2]);
      float ce = (d - hv) / hv;
      double cerr = ce;
      err += cerr * cerr;
    }
  }
  return err;
}

/* calcScoreHeatmapActiveRegion (LooperSolver.hpp:3583-3617). */
double orc_heatmap_score(int n, const float *pos, const float *heat, int diag,
                         int n_bounds, const int *bounds, int moved) {
  if (moved >= 0)
    return hm_local(n, pos, heat, diag, n_bounds, bounds, moved);
  double err = 0.0;
  for (int i = 0; i < n; ++i)
    err += hm_local(n, pos, heat, diag, n_bounds, bounds, i);
  return err;
}

/* MonteCarloHeatmap (LooperSolver.hpp:1424-1565). */
void orc_heatmap_anneal(int n, float *pos, const unsigned char *fixed,
                        const float *heat, int diag, int n_bounds,
                        const int *bounds, const orc_params *p,
                        float step_size, int incremental, orc_rng *rng,
                        orc_result *res) {
  memset(res, 0, sizeof(*res));
  step_size *= 0.5;
  if (n <= 1)
    return;
  rng_ctx c;
  rng_begin(&c, rng, n, fixed);
  int philox = rng->kind == ORC_RNG_PHILOX;
  double T = p->max_temp, tp;
  double score_curr = orc_heatmap_score(n, pos, heat, diag, n_bounds, bounds, -1);
  int sph = p->sphere_radius > 0.0f;
  double boundary_sum = 0.0;
  if (sph) {
    for (int k = 0; k < n; ++k)
      boundary_sum += sphere_pen(pos + 3 * k, p->sphere_radius);
    score_curr += boundary_sum;
  }
  double score_prev = score_curr, milestone_score = score_curr;
  int64_t success = 0, milestone_success = 0, i = 1;
  if (score_curr != score_curr || score_curr < 1e-6 ||
      (philox && c.n_movable == 0)) {
    res->score = 0.0;
    rng_end(&c);
    return;
  }
  for (;;) {
    int pb = draw_bead(&c, n);
    res->proposals++;
    if (fixed && fixed[pb])
      continue;
    float *q = pos + 3 * pb;
    double old_pen = 0.0, before = 0.0;
    if (sph)
      old_pen = sphere_pen(q, p->sphere_radius);
    if (incremental)
      before = hm_local(n, pos, heat, diag, n_bounds, bounds, pb);
    float d[3], old[3] = {q[0], q[1], q[2]};
    draw_disp(&c, step_size, p->use2d, d);
    q[0] += d[0];
    q[1] += d[1];
    q[2] += d[2];
    if (incremental) {
      double after = hm_local(n, pos, heat, diag, n_bounds, bounds, pb);
      score_curr = (score_prev - (sph ? boundary_sum : 0.0)) + 2.0 * (after - before);
    } else {
      score_curr = orc_heatmap_score(n, pos, heat, diag, n_bounds, bounds, -1);
    }
    if (sph) {
      double new_pen = sphere_pen(q, p->sphere_radius);
      score_curr += boundary_sum - old_pen + new_pen;
    }
    int ok = score_curr <= score_prev;
    if (!ok && T > 0.0) {
      tp = p->jump_scale * exp(-p->jump_coef * (score_curr / score_prev) / T);
      ok = draw_chance(&c, (float)tp);
    }
    if (ok) {
      success++;
      milestone_success++;
      if (sph) {
        double new_pen = sphere_pen(q, p->sphere_radius);
        boundary_sum = boundary_sum - old_pen + new_pen;
      }
    } else {
      if (philox) {
        q[0] = old[0];
        q[1] = old[1];
        q[2] = old[2];
      } else {
        q[0] -= d[0];
        q[1] -= d[1];
        q[2] -= d[2];
      }
      score_curr = score_prev;
    }
    end_move(&c);
    T *= p->dt_temp;
    if (i % p->milestone_steps == 0) {
      if ((score_curr > p->improvement * milestone_score &&
           milestone_success < p->min_successes) ||
          score_curr < 1e-6)
        break;
      milestone_score = score_curr;
      milestone_success = 0;
    }
    if (p->max_moves > 0 && i >= p->max_moves)
      break;
    score_prev = score_curr;
    i++;
  }
  res->score = score_curr;
  res->moves = i;
  res->accepted = success;
  rng_end(&c);
}

/* ------------------------------------------------------------------ */
/* Subanchor smoothing                                                 */
/* ------------------------------------------------------------------ */
static double bond_term(const float *a, const float *b, double dtn,
                        const orc_params *p) {
  if (dtn < 1e-6)
    dtn = 1e-6;
  float len = v_len(a[0] - b[0], a[1] - b[1], a[2] - b[2]);
  double diff = (len - dtn) / dtn;
  return diff * diff * (diff >= 0.0f ? p->k_stretch : p->k_squeeze);
}

/* calcScoreStructureSmooth(true, true) (LooperSolver.hpp:3414-3451). */
static double smooth_structure(int n, const float *pos, const double *dtn,
                               const orc_params *p) {
  double sca = 0.0, scb = 0.0;
  float v2[3] = {0, 0, 0};
  for (int i = 0; i + 1 < n; ++i) {
    const float *a = pos + 3 * i, *b = pos + 3 * (i + 1);
    float v[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
    sca += bond_term(a, b, dtn[i], p);
    if (i > 0) {
      double ang = v_angle(v, v2);
      scb += ang * ang * ang * p->k_angle;
    }
    v2[0] = v[0];
    v2[1] = v[1];
    v2[2] = v[2];
  }
  return sca * p->w_dist + scb * p->w_angle;
}

double orc_smooth_full_score(int n, const float *pos, const double *dist_to_next,
                             const orc_params *p) {
  double sc = smooth_structure(n, pos, dist_to_next, p);
  if (p->sphere_radius > 0.0f)
    for (int k = 0; k < n; ++k)
      sc += sphere_pen(pos + 3 * k, p->sphere_radius);
  return sc;
}

/* calcScoreStructureSmooth(moved, true, true) (LooperSolver.hpp:3453-3495). */
static double smooth_local(int n, const float *pos, const double *dtn,
                           const orc_params *p, int moved) {
  double sca = 0.0, scb = 0.0;
  float v2[3] = {0, 0, 0};
  for (int i = moved - 2; i < moved + 2; i++) {
    if (i < 0 || i + 1 >= n)
      continue;
    const float *a = pos + 3 * i, *b = pos + 3 * (i + 1);
    float v[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
    if (i == moved - 1 || i == moved)
      sca += bond_term(a, b, dtn[i], p);
    if (i > moved - 2 && i > 0) {
      double ang = v_angle(v, v2);
      scb += ang * ang * ang * p->k_angle;
    }
    v2[0] = v[0];
    v2[1] = v[1];
    v2[2] = v[2];
  }
  return sca + scb;
}

double orc_smooth_local_score(int n, const float *pos,
                              const double *dist_to_next, const orc_params *p,
                              int moved) {
  double sc = smooth_local(n, pos, dist_to_next, p, moved);
  if (p->sphere_radius > 0.0f)
    sc += sphere_pen(pos + 3 * moved, p->sphere_radius);
  return sc;
}

/* Extended arc energy: the bond and angle terms above with one target and
 * the extension's constants, weights 1. */
static orc_params ext_params(const orc_ext *x) {
  orc_params q;
  memset(&q, 0, sizeof(q));
  q.k_stretch = x->k_stretch;
  q.k_squeeze = x->k_squeeze;
  q.k_angle = x->k_angle;
  q.w_dist = 1.0f;
  q.w_angle = 1.0f;
  return q;
}

static double ext_target(const orc_ext *x) {
  return x->bond_target < 1e-5 ? 1e-5 : x->bond_target;
}

static double ext_full(int n, const float *pos, const orc_ext *x) {
  const orc_params q = ext_params(x);
  const double t = ext_target(x);
  double sca = 0.0, scb = 0.0;
  float v2[3] = {0, 0, 0};
  for (int i = 0; i + 1 < n; ++i) {
    const float *a = pos + 3 * i, *b = pos + 3 * (i + 1);
    float v[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
    sca += bond_term(a, b, t, &q);
    if (i > 0) {
      double ang = v_angle(v, v2);
      scb += ang * ang * ang * q.k_angle;
    }
    v2[0] = v[0];
    v2[1] = v[1];
    v2[2] = v[2];
  }
  return sca + scb;
}

static double ext_local(int n, const float *pos, const orc_ext *x, int moved) {
  const orc_params q = ext_params(x);
  const double t = ext_target(x);
  double sca = 0.0, scb = 0.0;
  float v2[3] = {0, 0, 0};
  for (int i = moved - 2; i < moved + 2; i++) {
    if (i < 0 || i + 1 >= n)
      continue;
    const float *a = pos + 3 * i, *b = pos + 3 * (i + 1);
    float v[3] = {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
    if (i == moved - 1 || i == moved)
      sca += bond_term(a, b, t, &q);
    if (i > moved - 2 && i > 0) {
      double ang = v_angle(v, v2);
      scb += ang * ang * ang * q.k_angle;
    }
    v2[0] = v[0];
    v2[1] = v[1];
    v2[2] = v[2];
  }
  return sca + scb;
}

double orc_arcs_ext_score(int n, const float *pos, const orc_ext *x, int moved) {
  return moved < 0 ? ext_full(n, pos, x) : ext_local(n, pos, x, moved);
}

/* MonteCarloArcsSmooth (LooperSolver.hpp:4798-5047), orientation and
 * subanchor-heatmap terms off.
 *
 * ORC_SCHEDULE_GPU restates the schedule of the reference's smoothing kernel
 * (MonteCarloSmoothKernelMultiWarp, src/ParallelMonteCarloSmooth.cu:258-337):
 * blocks of 256 moves while fewer than milestone_steps moves are done
 * (:267-269,317), so exactly milestone_steps rounded up to 256 moves (none
 * when it is <= 0).  Its milestone test (:320-335) runs only when
 * iterations % milestone_steps < 256, which inside that loop happens only
 * after the last block, so it never shortens the chain and is not restated.
 * An uphill move is tested against
 * scale * exp(-coef * (E_new / max(E_prev, 1e-12)) / T) when T > 0 (:291-296).
 * res->best is the lowest running score of the chain (:299-301), by which the
 * reference's host picks the reported warp (:462-472). */
void orc_smooth_anneal(int n, float *pos, const unsigned char *fixed,
                       const double *dist_to_next, const orc_params *p,
                       float step_size, orc_rng *rng, orc_result *res) {
  memset(res, 0, sizeof(*res));
  rng_ctx c;
  rng_begin(&c, rng, n, fixed);
  c.u_from_bead = 1; /* smoothing: one Philox block a move */
  int philox = rng->kind == ORC_RNG_PHILOX;
  double T = p->max_temp, dt = p->dt_temp, tp;
  double curr_structure = orc_smooth_full_score(n, pos, dist_to_next, p);
  double prev_structure = curr_structure;
  double score_curr = curr_structure + 0.0 + 0.0;
  double score_prev = score_curr, milestone_score = score_curr;
  int64_t success = 0, milestone_success = 0, i = 1;
  int gpu = p->schedule == ORC_SCHEDULE_GPU;
  int64_t cap = p->milestone_steps > 0 ? ((int64_t)p->milestone_steps + 255) / 256 * 256 : 0;
  res->best = score_curr;
  if ((philox && c.n_movable == 0) || (gpu && cap == 0)) {
    res->score = score_curr;
    rng_end(&c);
    return;
  }
  for (;;) {
    int pb = draw_bead(&c, n);
    res->proposals++;
    if (fixed && fixed[pb])
      continue;
    float *q = pos + 3 * pb;
    double lp = orc_smooth_local_score(n, pos, dist_to_next, p, pb);
    float d[3], old[3] = {q[0], q[1], q[2]};
    draw_disp(&c, step_size, p->use2d, d);
    q[0] += d[0];
    q[1] += d[1];
    q[2] += d[2];
    double lc = orc_smooth_local_score(n, pos, dist_to_next, p, pb);
    curr_structure = curr_structure - lp + lc;
    score_curr = curr_structure + 0.0 + 0.0;
    int ok = score_curr < score_prev;
    if (!ok && T > 0.0) {
      double den = gpu && score_prev < 1e-12 ? 1e-12 : score_prev;
      tp = p->jump_scale * exp(-p->jump_coef * (score_curr / den) / T);
      ok = draw_chance(&c, (float)tp);
    }
    if (ok) {
      success++;
      milestone_success++;
      score_prev = score_curr;
      prev_structure = curr_structure;
      if (score_curr < res->best) res->best = score_curr;
    } else {
      if (philox) {
        q[0] = old[0];
        q[1] = old[1];
        q[2] = old[2];
      } else {
        q[0] -= d[0];
        q[1] -= d[1];
        q[2] -= d[2];
      }
      score_curr = score_prev;
      curr_structure = prev_structure;
    }
    end_move(&c);
    if (gpu) {
      if (i >= cap) break;
    } else if (i % p->milestone_steps == 0) {
      if ((score_curr > p->improvement * milestone_score &&
           milestone_success < p->min_successes) ||
          score_curr < 1e-6)
        break;
      milestone_score = score_curr;
      milestone_success = 0;
    }
    T *= dt;
    if (p->max_moves > 0 && i >= p->max_moves)
      break;
    i++;
  }
  res->score = score_curr;
  res->moves = i;
  res->accepted = success;
  rng_end(&c);
}

/* ------------------------------------------------------------------ */
/* Arc marking: InteractionArcs::markArcs (InteractionArcs.hpp:207-336) */
/* ------------------------------------------------------------------ */
typedef struct {
  int start, end, gstart, gend, score, eff, factor;
  int order; /* input position: ties keep input order */
} arc_t;

/* InteractionArc::operator< (InteractionArc.hpp:74-84): start, end, factor. */
static int arc_cmp(const void *x, const void *y) {
  const arc_t *a = (const arc_t *)x, *b = (const arc_t *)y;
  if (a->start != b->start)
    return a->start < b->start ? -1 : 1;
  if (a->end != b->end)
    return a->end < b->end ? -1 : 1;
  if (a->factor != b->factor)
    return a->factor < b->factor ? -1 : 1;
  return a->order < b->order ? -1 : (a->order > b->order);
}

static int emit(int *out, int cap, int *cnt, const arc_t *a) {
  if (*cnt < cap) {
    int *o = out + 7 * (*cnt);
    o[0] = a->start;
    o[1] = a->end;
    o[2] = a->gstart;
    o[3] = a->gend;
    o[4] = a->score;
    o[5] = a->eff;
    o[6] = a->factor;
  }
  (*cnt)++;
  return 0;
}

/* Flush the arcs gathered for one start anchor: tmp_arcs is a std::map keyed
 * by the end anchor, iterated in ascending key order (:263-316). */
static void flush_group(arc_t *g, int ng, int *out, int cap, int *cnt) {
  /* order by end anchor (std::map key), keeping arrival order within a key */
  for (int a = 1; a < ng; ++a) { /* insertion sort: stable */
    arc_t x = g[a];
    int b = a - 1;
    while (b >= 0 && g[b].end > x.end) {
      g[b + 1] = g[b];
      b--;
    }
    g[b + 1] = x;
  }
  int s = 0;
  while (s < ng) {
    int e = s;
    while (e < ng && g[e].end == g[s].end)
      e++;
    int sz = e - s;
    arc_t *el = g + s;
    if (sz == 1) {
      emit(out, cap, cnt, &el[0]);
    } else {
      /* std::sort by (start, end, factor); equal keys keep arrival order */
      qsort(el, sz, sizeof(arc_t), arc_cmp);
      int multiple = 0;
      for (int j = 1; j < sz; ++j)
        if (el[j].factor != el[j - 1].factor)
          multiple = 1;
      int total = 0, fscore = 0, first = 0;
      for (int j = 0; j <= sz; ++j) {
        if (j == sz || (j > 0 && el[j].factor != el[j - 1].factor)) {
          arc_t r = el[first];
          r.score = fscore;
          r.eff = multiple ? 0 : fscore;
          emit(out, cap, cnt, &r);
          first = j;
          total += fscore;
          fscore = 0;
        }
        if (j < sz)
          fscore += el[j].score;
      }
      if (multiple) {
        /* InteractionArc(start, end, 0, -1) with eff_score = total */
        arc_t r;
        r.start = el[0].start;
        r.end = el[0].end;
        r.gstart = -1;
        r.gend = -1;
        r.score = 0;
        r.eff = total;
        r.factor = -1;
        emit(out, cap, cnt, &r);
      }
    }
    s = e;
  }
}

int orc_mark_arcs(int n_anchors, const int *a_start, const int *a_end,
                  int n_raw, const int *r_start, const int *r_end,
                  const int *r_score, const int *r_factor, int *out, int cap,
                  int *non_matching) {
  arc_t *raw = (arc_t *)malloc(sizeof(arc_t) * (n_raw > 0 ? n_raw : 1));
  arc_t *grp = (arc_t *)malloc(sizeof(arc_t) * (n_raw > 0 ? n_raw : 1));
  for (int i = 0; i < n_raw; ++i) {
    raw[i].start = r_start[i];
    raw[i].end = r_end[i];
    raw[i].score = r_score[i];
    raw[i].factor = r_factor[i];
    raw[i].order = i;
  }
  qsort(raw, n_raw, sizeof(arc_t), arc_cmp);
  int cnt = 0, ng = 0, nm = 0, last_start = -1;
  for (int i = 0; i <= n_raw; ++i) {
    int st = -1, en = -1;
    if (i < n_raw) {
      /* every anchor of length > 1 that contains the position; last wins
       * (Anchor::length / contains, Anchor.hpp:81-87) */
      for (int j = 0; j < n_anchors; ++j) {
        int len = (a_start[j] == 0 && a_end[j] == 0) ? 0 : a_end[j] - a_start[j] + 1;
        if (len > 1) {
          if (raw[i].start >= a_start[j] && raw[i].start <= a_end[j])
            st = j;
          if (raw[i].end >= a_start[j] && raw[i].end <= a_end[j])
            en = j;
        }
      }
      if (st == -1 || en == -1) {
        ++nm;
        continue;
      }
      if (st == en)
        continue;
    }
    if (st != last_start || i == n_raw) {
      flush_group(grp, ng, out, cap, &cnt);
      ng = 0;
      last_start = st;
    }
    if (i < n_raw) {
      arc_t a;
      a.start = st;
      a.end = en;
      a.gstart = raw[i].start;
      a.gend = raw[i].end;
      a.score = raw[i].score;
      a.eff = raw[i].score;
      a.factor = raw[i].factor;
      a.order = ng;
      grp[ng++] = a;
    }
  }
  free(raw);
  free(grp);
  if (non_matching)
    *non_matching = nm;
  return cnt <= cap ? cnt : -cnt - 1;
}

/* ------------------------------------------------------------------ */
/* HCM lines                                                           */
/* ------------------------------------------------------------------ */
int orc_hcm_cluster_line(char *buf, int cap, int start, int end, char orient,
                         float x, float y, float z, int n_children,
                         const int *children) {
  int w = snprintf(buf, cap, "%d %d %c %f %f %f %zu", start, end, orient,
                   (double)x, (double)y, (double)z, (size_t)n_children);
  for (int i = 0; i < n_children; ++i)
    w += snprintf(buf + (w < cap ? w : cap), w < cap ? cap - w : 0, " %d",
                  children[i]);
  w += snprintf(buf + (w < cap ? w : cap), w < cap ? cap - w : 0, "\n");
  return w;
}

int orc_hcm_arc_line(char *buf, int cap, const int a[7]) {
  return snprintf(buf, cap, "%d %d %d %d %d %d %d\n", a[0], a[1], a[2], a[3],
                  a[4], a[5], a[6]);
}

/* ------------------------------------------------------------------ */
/* Replay of a kernel trace (test infrastructure)                      */
/* ------------------------------------------------------------------ */
typedef double (*local_fn)(void *ctx, const float *pos, int moved);

typedef struct {
  int n;
  const float *exp_dist;
  const loop_ent *loops;
  int m;
  const orc_params *p;
  const double *dtn;
  const float *heat;
  int diag, n_bounds;
  const int *bounds;
  const orc_ext *ext;
} replay_ctx;

static double arcs_local_cb(void *vc, const float *pos, int moved) {
  replay_ctx *c = (replay_ctx *)vc;
  double sc = arcs_dist_local(c->n, pos, c->exp_dist, c->p, moved) +
              loop_energy(pos, c->loops, c->m, moved);
  if (c->p->sphere_radius > 0.0f)
    sc += sphere_pen(pos + 3 * moved, c->p->sphere_radius);
  if (c->ext)
    sc += ext_local(c->n, pos, c->ext, moved);
  return sc;
}

static double smooth_local_cb(void *vc, const float *pos, int moved) {
  replay_ctx *c = (replay_ctx *)vc;
  return orc_smooth_local_score(c->n, pos, c->dtn, c->p, moved);
}

static double heat_local_cb(void *vc, const float *pos, int moved) {
  replay_ctx *c = (replay_ctx *)vc;
  return hm_local(c->n, pos, c->heat, c->diag, c->n_bounds, c->bounds, moved);
}

/* Relative distance of a from the threshold b (for the stop margin). */
static double rel_gap(double a, double b) {
  double s = fabs(b) > 0.0 ? fabs(b) : 1.0;
  return fabs(a - b) / s;
}

/* The milestone predicate of `kind` under p->schedule at counted move i,
 * with the running energy E, the milestone energy *E_ms and the successes
 * since it; updates the milestone state and returns 1 when the annealer
 * stops after move i.  CPU schedule: MonteCarloArcs :4765-4783,
 * MonteCarloHeatmap :1543-1553, MonteCarloArcsSmooth :5015-5034; GPU
 * schedule: ParallelMonteCarloArcs.cu:631-655 (arcs),
 * ParallelMonteCarloSmooth.cu:267-317 (smoothing: the cap alone). */
static int schedule_stop(int kind, const orc_params *p, int64_t i, double E,
                         double *E_ms, int64_t *succ, int *misses, double *margin) {
  int gpu = p->schedule == ORC_SCHEDULE_GPU && kind != 1;
  int stop = 0;
  if (gpu && kind == 2) {
    int64_t cap = p->milestone_steps > 0 ? ((int64_t)p->milestone_steps + 255) / 256 * 256 : 0;
    stop = i >= cap;
  } else if (gpu) {
    if (i % 256 == 0) {
      int64_t cap = p->milestone_steps > 0 ? ((int64_t)p->milestone_steps + 255) / 256 * 256 : 0;
      int slow = *succ < p->min_successes;
      int guard = *E_ms > 1e-10;
      int miss = (E > p->improvement * *E_ms && slow) || E < 1e-5 ||
                 (guard && E / *E_ms > 0.9999);
      if (slow) *margin = fmin(*margin, rel_gap(E, p->improvement * *E_ms));
      if (guard) *margin = fmin(*margin, rel_gap(E / *E_ms, 0.9999));
      *margin = fmin(*margin, rel_gap(E, 1e-5));
      *misses = miss ? *misses + 1 : 0;
      stop = *misses >= p->milestone_fails || E < 1e-5 || i >= cap;
      *E_ms = E;
      *succ = 0;
    }
  } else if (p->milestone_steps > 0 && i % p->milestone_steps == 0) {
    double floor = kind == 0 ? 1e-5 : 1e-6;
    int slow = *succ < p->min_successes;
    int miss = (E > p->improvement * *E_ms && slow) || E < floor;
    if (kind == 0) miss = miss || E / *E_ms > 0.9999;
    if (slow) *margin = fmin(*margin, rel_gap(E, p->improvement * *E_ms));
    if (kind == 0) *margin = fmin(*margin, rel_gap(E / *E_ms, 0.9999));
    *margin = fmin(*margin, rel_gap(E, floor));
    stop = miss;
    *E_ms = E;
    *succ = 0;
  }
  if (!stop && p->max_moves > 0 && i >= p->max_moves) stop = 1;
  return stop;
}

/* kind: 0 arcs (<=; CPU schedule: no T check, GPU schedule: T > 0 and
 * E > 0), 1 heatmap (<=, T>0, delta counted twice), 2 smoothing (strict <,
 * T>0; GPU schedule: the ratio's denominator at least 1e-12). */
static void replay_core(int kind, void *ctx, local_fn fn, int n, float *pos,
                        const unsigned char *fixed, const orc_params *p,
                        float step, double E, uint64_t seed, uint32_t chain,
                        int n_moves, const int *bead, const float *disp,
                        const int *gpu_acc, orc_replay_out *out) {
  orc_rng r;
  r.kind = ORC_RNG_PHILOX;
  r.seed = seed;
  r.chain = chain;
  r.move = 0;
  rng_ctx c;
  rng_begin(&c, &r, n, fixed);
  double T = p->max_temp;
  int gpu = p->schedule == ORC_SCHEDULE_GPU;
  double E_ms = E;
  int64_t succ = 0;
  int misses = 0;
  out->proposal_mismatch = 0;
  out->stop_at = -1;
  out->stop_margin = 1e300;
  for (int k = 0; k < n_moves; ++k) {
    int b = draw_bead(&c, n);
    float d[3];
    draw_disp(&c, step, p->use2d, d);
    if (b != bead[k] || d[0] != disp[3 * k] || d[1] != disp[3 * k + 1] ||
        d[2] != disp[3 * k + 2])
      out->proposal_mismatch++;
    b = bead[k];
    float *q = pos + 3 * b;
    float old[3] = {q[0], q[1], q[2]};
    double before = fn(ctx, pos, b);
    q[0] += disp[3 * k];
    q[1] += disp[3 * k + 1];
    q[2] += disp[3 * k + 2];
    double after = fn(ctx, pos, b);
    double dE = (kind == 1 ? 2.0 : 1.0) * (after - before);
    if (kind == 1 && p->sphere_radius > 0.0f)
      dE += sphere_pen(q, p->sphere_radius) - sphere_pen(old, p->sphere_radius);
    double En = E + dE;
    int ok = kind == 2 ? En < E : En <= E;
    uint32_t o[4];
    philox_block(&r, 1u, o);
    /* smoothing draws one block a move: its uniform is the bead draw's
       fractional part */
    float u = kind == 2 ? c.bead_u : orc_u01(o[0]);
    int test = kind == 0 ? (!gpu || (T > 0.0 && E > 0.0)) : T > 0.0;
    if (!ok && test) {
      double den = (kind == 2 && gpu && E < 1e-12) ? 1e-12 : E;
      double tp = p->jump_scale * exp(-p->jump_coef * (En / den) / T);
      ok = u < (float)tp;
    }
    /* distance of the decision from its threshold, in log-ratio units */
    double thr = (T > 0.0 && u > 0.0f) ? -T * log((double)u / p->jump_scale) / p->jump_coef : 0.0;
    double margin = (E > 0.0 && En > 0.0 && thr > 0.0) ? fabs(log(En / E) - log(thr)) : 1e300;
    if (dE <= 0.0 && kind != 2) margin = fabs(dE) / (fabs(E) > 0 ? fabs(E) : 1.0);
    if (kind == 2 && dE < 0.0) margin = fabs(dE) / (fabs(E) > 0 ? fabs(E) : 1.0);
    out->before[k] = before;
    out->after[k] = after;
    out->orc_acc[k] = ok;
    out->margin[k] = margin;
    if (gpu_acc[k]) {
      E = En;
      succ++;
    } else {
      q[0] = old[0];
      q[1] = old[1];
      q[2] = old[2];
    }
    if (out->stop_at < 0 &&
        schedule_stop(kind, p, (int64_t)k + 1, E, &E_ms, &succ, &misses, &out->stop_margin))
      out->stop_at = (int64_t)k + 1;
    r.move++;
    T *= p->dt_temp;
  }
  out->final_energy = E;
  rng_end(&c);
}

void orc_arcs_replay(int n, const float *pos0, const unsigned char *fixed,
                     const float *exp_dist, int n_loops, const int *loop_i,
                     const int *loop_j, const float *loop_k,
                     const float *loop_r0, const orc_params *p,
                     float step_size, uint64_t seed, uint32_t chain,
                     int n_moves, const int *bead, const float *disp,
                     const int *gpu_acc, orc_replay_out *out) {
  orc_arcs_replay_ext(n, pos0, fixed, exp_dist, n_loops, loop_i, loop_j, loop_k, loop_r0, p,
                      NULL, step_size, seed, chain, n_moves, bead, disp, gpu_acc, out);
}

void orc_arcs_replay_ext(int n, const float *pos0, const unsigned char *fixed,
                         const float *exp_dist, int n_loops, const int *loop_i,
                         const int *loop_j, const float *loop_k,
                         const float *loop_r0, const orc_params *p,
                         const orc_ext *x, float step_size, uint64_t seed,
                         uint32_t chain, int n_moves, const int *bead,
                         const float *disp, const int *gpu_acc,
                         orc_replay_out *out) {
  int m;
  loop_ent *e = build_loops(n, n_loops, loop_i, loop_j, loop_k, loop_r0, &m);
  float *pos = (float *)malloc(sizeof(float) * 3 * (n > 0 ? n : 1));
  memcpy(pos, pos0, sizeof(float) * 3 * n);
  replay_ctx c = {n, exp_dist, e, m, p, NULL, NULL, 0, 0, NULL, x};
  double E = arcs_dist_full(n, pos, exp_dist, p, 1, 1) + loop_energy(pos, e, m, -1);
  if (p->sphere_radius > 0.0f)
    for (int k = 0; k < n; ++k) E += sphere_pen(pos + 3 * k, p->sphere_radius);
  if (x)
    E += ext_full(n, pos, x);
  replay_core(0, &c, arcs_local_cb, n, pos, fixed, p, step_size, E, seed, chain,
              n_moves, bead, disp, gpu_acc, out);
  free(pos);
  free(e);
}

void orc_smooth_replay(int n, const float *pos0, const unsigned char *fixed,
                       const double *dist_to_next, const orc_params *p,
                       float step_size, uint64_t seed, uint32_t chain,
                       int n_moves, const int *bead, const float *disp,
                       const int *gpu_acc, orc_replay_out *out) {
  float *pos = (float *)malloc(sizeof(float) * 3 * (n > 0 ? n : 1));
  memcpy(pos, pos0, sizeof(float) * 3 * n);
  replay_ctx c = {n, NULL, NULL, 0, p, dist_to_next, NULL, 0, 0, NULL, NULL};
  double E = orc_smooth_full_score(n, pos, dist_to_next, p);
  replay_core(2, &c, smooth_local_cb, n, pos, fixed, p, step_size, E, seed, chain,
              n_moves, bead, disp, gpu_acc, out);
  free(pos);
}

void orc_heatmap_replay(int n, const float *pos0, const unsigned char *fixed,
                        const float *heat, int diag, int n_bounds,
                        const int *bounds, const orc_params *p,
                        float step_size, uint64_t seed, uint32_t chain,
                        int n_moves, const int *bead, const float *disp,
                        const int *gpu_acc, orc_replay_out *out) {
  float *pos = (float *)malloc(sizeof(float) * 3 * (n > 0 ? n : 1));
  memcpy(pos, pos0, sizeof(float) * 3 * n);
  replay_ctx c = {n, NULL, NULL, 0, p, NULL, heat, diag, n_bounds, bounds, NULL};
  double E = orc_heatmap_score(n, pos, heat, diag, n_bounds, bounds, -1);
  if (p->sphere_radius > 0.0f)
    for (int k = 0; k < n; ++k) E += sphere_pen(pos + 3 * k, p->sphere_radius);
  replay_core(1, &c, heat_local_cb, n, pos, fixed, p, step_size * 0.5f, E, seed, chain,
              n_moves, bead, disp, gpu_acc, out);
  free(pos);
}

/* ------------------------------------------------------------------ */
/* anchor-level expected distances (LooperSolver.hpp:5494-5627)       */
/* ------------------------------------------------------------------ */

/* freqToDistance(freq, memo = true) (LooperSolver.hpp:3949-3967): the int
 * count plus the float shift is a float; the rest is FP64. */
static float orc_freq_to_distance(int freq, const float *memo, float a,
                                  float scale, float shift, float base) {
  if (freq >= 1 && freq <= 100)
    return memo[freq];
  if (a < 0.0f) {
    int fi = (int)((float)freq + shift);
    if (fi < 1)
      fi = 1;
    return (float)((double)base + (double)scale * pow((double)fi, (double)a));
  }
  return (float)((double)base +
                 (double)scale / exp((double)a * (double)((float)freq + shift)));
}

/* std::map<int, int> as a sorted array: lookup, and operator[] inserting 0. */
typedef struct {
  int *key, *val;
  int n, cap;
} orc_imap;

static int orc_imap_find(const orc_imap *m, int k) {
  int lo = 0, hi = m->n;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (m->key[mid] < k)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

static int *orc_imap_at(orc_imap *m, int k) {
  int p = orc_imap_find(m, k);
  if (p < m->n && m->key[p] == k)
    return &m->val[p];
  if (m->n == m->cap) {
    m->cap = m->cap ? 2 * m->cap : 64;
    m->key = (int *)realloc(m->key, sizeof(int) * m->cap);
    m->val = (int *)realloc(m->val, sizeof(int) * m->cap);
  }
  memmove(m->key + p + 1, m->key + p, sizeof(int) * (m->n - p));
  memmove(m->val + p + 1, m->val + p, sizeof(int) * (m->n - p));
  m->key[p] = k;
  m->val[p] = 0;
  m->n++;
  return &m->val[p];
}

int orc_anchor_targets(int n, const int *active, const int *arc_ptr,
                       const int *arc_idx, const int *arc_start,
                       const int *arc_end, const int *arc_score, int n_long,
                       const int *long_start, const int *long_end,
                       const int *long_score, int n_anc, const int *anc_start,
                       const int *anc_end, int first_cluster,
                       const float *memo, float count_a, float count_scale,
                       float count_shift, float count_base, const float *heat,
                       float influence, float *dense, long long *stats4) {
  int i, j, k, rc = 0;
  orc_imap m = {NULL, NULL, 0, 0};
  for (k = 0; k < 4; ++k)
    stats4[k] = 0;
  /* init(n), add(-1), clearDiagonal(1) */
  for (i = 0; i < n; ++i)
    for (j = 0; j < n; ++j)
      dense[(size_t)i * n + j] = i == j ? 0.0f : -1.0f;
  for (i = 0; i < n; ++i)
    *orc_imap_at(&m, active[i]) = i;
  /* the arcs of the active clusters, forward only (:5512-5539) */
  for (i = 0; i < n && rc == 0; ++i) {
    int ai = active[i];
    for (k = arc_ptr[i]; k < arc_ptr[i + 1]; ++k) {
      int arc = arc_idx[k], other, a, b;
      float e;
      if (arc_start[arc] == ai)
        other = arc_end[arc];
      else if (arc_end[arc] == ai)
        other = arc_start[arc];
      else {
        rc = -1;
        break;
      }
      if (other < ai)
        continue;
      e = (float)(double)orc_freq_to_distance(arc_score[arc], memo, count_a,
                                              count_scale, count_shift,
                                              count_base);
      a = *orc_imap_at(&m, ai);
      b = *orc_imap_at(&m, other);
      dense[(size_t)a * n + b] = e;
      dense[(size_t)b * n + a] = e;
    }
  }
  /* long arcs: linear anchor scan, slots through the same map (:5547-5588) */
  if (rc == 0 && n_long > 0 && n_anc > 0) {
    int *anc_to_active = (int *)malloc(sizeof(int) * n_anc);
    for (i = 0; i < n_anc; ++i)
      anc_to_active[i] = -1;
    for (i = 0; i < m.n; ++i)
      if (m.key[i] >= first_cluster && m.key[i] < first_cluster + n_anc)
        anc_to_active[m.key[i] - first_cluster] = m.val[i];
    for (k = 0; k < n_long; ++k) {
      int ia = -1, ib = -1, a, b;
      for (i = 0; i < n_anc; ++i)
        if (long_start[k] >= anc_start[i] && long_start[k] <= anc_end[i]) {
          ia = i;
          break;
        }
      for (i = 0; i < n_anc; ++i)
        if (long_end[k] >= anc_start[i] && long_end[k] <= anc_end[i]) {
          ib = i;
          break;
        }
      if (ia < 0 || ib < 0 || ia == ib) {
        stats4[1]++;
        continue;
      }
      a = anc_to_active[ia];
      b = anc_to_active[ib];
      if (a < 0 || b < 0) {
        stats4[2]++;
        continue;
      }
      if (dense[(size_t)a * n + b] >= 0.0f) {
        stats4[3]++;
        continue;
      }
      {
        float ed = orc_freq_to_distance(long_score[k], memo, count_a,
                                        count_scale, count_shift, count_base);
        dense[(size_t)a * n + b] = ed;
        dense[(size_t)b * n + a] = ed;
        stats4[0]++;
      }
    }
    free(anc_to_active);
  }
  /* the anchor heatmap's influence (:5598-5625): getDiagonalSize, getRange */
  if (rc == 0 && heat && n > 0) {
    int w, diag = 0, found = 0;
    float max_val = 0.0f;
    for (w = 0; w < n && !found; ++w)
      for (i = 0; i + w < n; ++i)
        if ((double)heat[(size_t)i * n + i + w] > 1e-6) {
          diag = w;
          found = 1;
          break;
        }
    for (i = 0; i < n; ++i)
      for (j = i + diag; j < n; ++j)
        if (heat[(size_t)i * n + j] > max_val)
          max_val = heat[(size_t)i * n + j];
    if ((double)max_val > 1e-6)
      for (i = 0; i < n; ++i)
        for (j = i + 1; j < n; ++j) {
          float s;
          if (dense[(size_t)i * n + j] < 0.0f)
            continue;
          s = (heat[(size_t)i * n + j] / max_val) * influence;
          if (s > 1.0f)
            s = 1.0f;
          dense[(size_t)i * n + j] *= (1.0f - s);
          dense[(size_t)j * n + i] = dense[(size_t)i * n + j];
        }
  }
  free(m.key);
  free(m.val);
  return rc;
}

/* ------------------------------------------------------------------ */
/* stress refinement (LooperSolver.hpp:5638-5913)                     */
/* ------------------------------------------------------------------ */

/* freqToDistance(freq, memo = false) (LooperSolver.hpp:3949-3967). */
static float orc_freq_to_distance_formula(int freq, const orc_stress_params *p) {
  if (p->count_a < 0.0f) {
    int fi = (int)((float)freq + p->count_shift);
    if (fi < 1)
      fi = 1;
    return (float)((double)p->count_base +
                   (double)p->count_scale * pow((double)fi, (double)p->count_a));
  }
  return (float)((double)p->count_base +
                 (double)p->count_scale /
                     exp((double)p->count_a * (double)((float)freq + p->count_shift)));
}

/* genomicLengthToDistance (LooperSolver.hpp:3900-3904). */
static double orc_genomic_length_to_distance(int length, const orc_stress_params *p) {
  return (double)p->glen_base +
         (double)p->glen_scale * pow(length / 1000.0, (double)p->glen_power);
}

static void orc_merge_sort_idx(int *a, int *tmp, int n, const int *key) {
  int w, i;
  for (w = 1; w < n; w *= 2) {
    for (i = 0; i < n; i += 2 * w) {
      int lo = i, mid = i + w < n ? i + w : n, hi = i + 2 * w < n ? i + 2 * w : n;
      int x = lo, y = mid, k = lo;
      while (x < mid && y < hi)
        tmp[k++] = key[a[y]] < key[a[x]] ? a[y++] : a[x++];
      while (x < mid)
        tmp[k++] = a[x++];
      while (y < hi)
        tmp[k++] = a[y++];
    }
    memcpy(a, tmp, sizeof(int) * n);
  }
}

typedef struct {
  int i, j;
  float t, w;
} orc_pair;

/* The angle energy k * acos(c)^3 of the three beads around i (:5836-5845);
 * returns 0 with *ok = 0 when a bond is shorter than 1e-9. */
static float orc_stress_angle(const float *X, int i, float k, int *ok) {
  float v1[3], v2[3], n1, n2, c, th;
  int a;
  for (a = 0; a < 3; ++a) {
    v1[a] = X[3 * i + a] - X[3 * (i - 1) + a];
    v2[a] = X[3 * (i + 1) + a] - X[3 * i + a];
  }
  n1 = v_len(v1[0], v1[1], v1[2]);
  n2 = v_len(v2[0], v2[1], v2[2]);
  if (n1 < 1e-9f || n2 < 1e-9f) {
    *ok = 0;
    return 0.0f;
  }
  *ok = 1;
  c = (v1[0] * v2[0] + v1[1] * v2[1] + v1[2] * v2[2]) / (n1 * n2);
  if (c > 1.0f)
    c = 1.0f;
  if (c < -1.0f)
    c = -1.0f;
  th = acosf(c);
  return k * th * th * th;
}

int orc_stress_refine(int n, const int *active, const int *genomic_pos,
                      const float *pos, int n_arcs, const int *arc_start,
                      const int *arc_end, const int *arc_score, int n_long,
                      const int *long_start, const int *long_end,
                      const int *long_score, int n_anc, const int *anc_start,
                      const int *anc_end, int first_cluster,
                      const orc_stress_params *p, int max_iter, float lr,
                      int *order_out, float *pos_out, orc_stress_out *out) {
  int i, k, it, N = n;
  int *ord, *tmp, *gp, *anc_to_active, *seen;
  float *X, *G, *bb;
  orc_pair *pairs;
  long long np = 0, cap_pairs;
  int backbone_active;
  double prev_total = 1e300;
  float cur_lr = lr;
  memset(out, 0, sizeof(*out));
  out->lr = lr;
  for (i = 0; i < n; ++i)
    order_out[i] = active[i];
  memcpy(pos_out, pos, sizeof(float) * 3 * (size_t)n);
  if (max_iter <= 0 || n < 2)
    return 0;
  /* sort active_region by genomic position (:5647-5650) */
  ord = (int *)malloc(sizeof(int) * n);
  tmp = (int *)malloc(sizeof(int) * n);
  for (i = 0; i < n; ++i)
    ord[i] = i;
  orc_merge_sort_idx(ord, tmp, n, genomic_pos);
  gp = (int *)malloc(sizeof(int) * n);
  X = (float *)malloc(sizeof(float) * 3 * n);
  G = (float *)malloc(sizeof(float) * 3 * n);
  for (i = 0; i < n; ++i) {
    order_out[i] = active[ord[i]];
    gp[i] = genomic_pos[ord[i]];
    X[3 * i] = pos[3 * ord[i]];
    X[3 * i + 1] = pos[3 * ord[i] + 1];
    X[3 * i + 2] = pos[3 * ord[i] + 2];
  }
  anc_to_active = (int *)malloc(sizeof(int) * (n_anc > 0 ? n_anc : 1));
  for (i = 0; i < n_anc; ++i)
    anc_to_active[i] = -1;
  for (i = 0; i < N; ++i) {
    int ci = order_out[i];
    if (ci >= first_cluster && ci < first_cluster + n_anc)
      anc_to_active[ci - first_cluster] = i;
  }
  /* unique pair targets, first one wins (:5670-5729) */
  backbone_active = p->k_stretch > 1e-6f || p->k_squeeze > 1e-6f;
  seen = (int *)malloc(sizeof(int) * (size_t)N * N);
  for (k = 0; k < N * N; ++k)
    seen[k] = -1;
  cap_pairs = 1024;
  pairs = (orc_pair *)malloc(sizeof(orc_pair) * cap_pairs);
#define ORC_ADD_PAIR(AI, AJ, T)                                                \
  do {                                                                         \
    int ai_ = (AI), aj_ = (AJ);                                                \
    if (ai_ != aj_) {                                                          \
      if (ai_ > aj_) {                                                         \
        int s_ = ai_;                                                          \
        ai_ = aj_;                                                             \
        aj_ = s_;                                                              \
      }                                                                        \
      if (!(backbone_active && aj_ - ai_ <= 1) && seen[ai_ * N + aj_] < 0) {   \
        seen[ai_ * N + aj_] = (int)np;                                         \
        if (np == cap_pairs) {                                                 \
          cap_pairs *= 2;                                                      \
          pairs = (orc_pair *)realloc(pairs, sizeof(orc_pair) * cap_pairs);    \
        }                                                                      \
        pairs[np].i = ai_;                                                     \
        pairs[np].j = aj_;                                                     \
        pairs[np].t = (T);                                                     \
        pairs[np].w = 1.0f;                                                    \
        np++;                                                                  \
      }                                                                        \
    }                                                                          \
  } while (0)
  for (k = 0; k < n_arcs; ++k) {
    int a = arc_start[k], b = arc_end[k], ai, aj;
    float t;
    if (a < first_cluster || a >= first_cluster + n_anc)
      continue;
    if (b < first_cluster || b >= first_cluster + n_anc)
      continue;
    ai = anc_to_active[a - first_cluster];
    aj = anc_to_active[b - first_cluster];
    if (ai < 0 || aj < 0)
      continue;
    t = orc_freq_to_distance_formula(arc_score[k], p);
    if (t > 1e-6f)
      ORC_ADD_PAIR(ai, aj, t);
  }
  for (k = 0; k < n_long; ++k) {
    int ia = -1, ib = -1, as, bs;
    float t;
    for (i = 0; i < n_anc; ++i)
      if (long_start[k] >= anc_start[i] && long_start[k] <= anc_end[i]) {
        ia = i;
        break;
      }
    for (i = 0; i < n_anc; ++i)
      if (long_end[k] >= anc_start[i] && long_end[k] <= anc_end[i]) {
        ib = i;
        break;
      }
    if (ia < 0 || ib < 0)
      continue;
    as = anc_to_active[ia];
    bs = anc_to_active[ib];
    if (as < 0 || bs < 0)
      continue;
    t = orc_freq_to_distance_formula(long_score[k], p);
    if (t > 1e-6f)
      ORC_ADD_PAIR(as, bs, t);
  }
#undef ORC_ADD_PAIR
  free(seen);
  out->n_pairs = np;
  /* backbone targets from the genomic gaps (:5754-5762) */
  bb = (float *)malloc(sizeof(float) * N);
  for (i = 0; i < N; ++i)
    bb[i] = -1.0f;
  for (i = 0; i + 1 < N; ++i) {
    int gap = abs(gp[i + 1] - gp[i]);
    if (gap > 0)
      bb[i] = (float)orc_genomic_length_to_distance(gap, p);
  }
  /* gradient descent (:5786-5906) */
  for (it = 0; it < max_iter; ++it) {
    double e_back = 0.0, e_hic = 0.0, e_ang = 0.0, total;
    long long q;
    for (k = 0; k < 3 * N; ++k)
      G[k] = 0.0f;
    for (i = 0; i + 1 < N; ++i) {
      float t = bb[i], d[3], dlen, e, kk, g;
      if (t <= 1e-6f)
        continue;
      d[0] = X[3 * i] - X[3 * (i + 1)];
      d[1] = X[3 * i + 1] - X[3 * (i + 1) + 1];
      d[2] = X[3 * i + 2] - X[3 * (i + 1) + 2];
      dlen = v_len(d[0], d[1], d[2]);
      if (dlen < 1e-9f)
        dlen = 1e-9f;
      e = (dlen - t) / t;
      kk = e >= 0.0f ? p->k_stretch : p->k_squeeze;
      e_back += (double)kk * e * e;
      g = 2.0f * kk * (dlen - t) / (t * t * dlen);
      for (k = 0; k < 3; ++k) {
        float gv = d[k] * g;
        G[3 * i + k] += gv;
        G[3 * (i + 1) + k] -= gv;
      }
    }
    for (q = 0; q < np; ++q) {
      const orc_pair *pr = &pairs[q];
      float d[3], dlen, e, g;
      d[0] = X[3 * pr->i] - X[3 * pr->j];
      d[1] = X[3 * pr->i + 1] - X[3 * pr->j + 1];
      d[2] = X[3 * pr->i + 2] - X[3 * pr->j + 2];
      dlen = v_len(d[0], d[1], d[2]);
      if (dlen < 1e-9f)
        dlen = 1e-9f;
      e = (dlen - pr->t) / pr->t;
      e_hic += (double)pr->w * e * e;
      g = 2.0f * pr->w * (dlen - pr->t) / (pr->t * pr->t * dlen);
      for (k = 0; k < 3; ++k) {
        float gv = d[k] * g;
        G[3 * pr->i + k] += gv;
        G[3 * pr->j + k] -= gv;
      }
    }
    if (p->k_angular > 0.0f) {
      const float h = 1e-3f;
      for (i = 1; i + 1 < N; ++i) {
        int ok, bi, axis;
        float E0 = orc_stress_angle(X, i, p->k_angular, &ok);
        if (!ok)
          continue;
        e_ang += (double)E0;
        for (bi = 0; bi < 3; ++bi) {
          int b = i - 1 + bi;
          for (axis = 0; axis < 3; ++axis) {
            float saved = X[3 * b + axis], Ep;
            X[3 * b + axis] = saved + h;
            Ep = orc_stress_angle(X, i, p->k_angular, &ok);
            X[3 * b + axis] = saved;
            if (!ok)
              continue;
            G[3 * b + axis] += (Ep - E0) / h;
          }
        }
      }
    }
    total = e_back + e_hic + e_ang;
    out->iterations = it + 1;
    out->total = total;
    out->backbone = e_back;
    out->hic = e_hic;
    out->angular = e_ang;
    if (total > prev_total && it > 0) {
      cur_lr *= 0.5f;
      if (cur_lr < 1e-6f) {
        out->stop = 2;
        break;
      }
    }
    for (k = 0; k < 3 * N; ++k)
      X[k] -= cur_lr * G[k];
    if (prev_total - total < 1e-7 * (total > 1.0 ? total : 1.0) && it > 20) {
      out->stop = 1;
      break;
    }
    prev_total = total;
  }
  out->lr = cur_lr;
  memcpy(pos_out, X, sizeof(float) * 3 * (size_t)N);
  free(ord);
  free(tmp);
  free(gp);
  free(X);
  free(G);
  free(bb);
  free(anc_to_active);
  free(pairs);
  return 0;
}

/*
 * ORACLE -- test infrastructure only.  A plain-C restatement of the
 * reference's chaos-game buffer path, used by tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg as the checker.  The product never links,
 * loads or calls this file.
 *
 * Restates, step for step, with IEEE double arithmetic in the same operation
 * order as the reference (build with -ffp-contract=off):
 *   - Isaac<u64,4> (src/rng/isaac.hpp:45-362): init 93-131 with flag=false,
 *     gen 77-90, rngstep 146-153, mix 171-182, rngstep4 196-203, next 321-329,
 *     setSeed(u64) 267-271.  This is ISAAC-64 with a 16-word state (rparam
 *     4), not the published 256-word ISAAC-64, so public ISAAC test vectors
 *     do not apply; it is pinned by vectors produced by the reference itself.
 *   - FlameRNG (src/rng/flame_rng.hpp): randNum 67-87 (double, u64 words),
 *     randBool 61-64, randPoint 151-158.
 *   - Flame::getRandomXForm (src/types/flame.hpp:212-219).
 *   - XForm::applyIteration (src/types/xform.hpp:211-227) with
 *     Affine::apply_to (src/types/affine.hpp:104-110).
 *   - the variations of src/variations/variations.hpp (see or_variation()).
 *   - RenderIterator (src/renderers/render_iterator.hpp:52-139) and
 *     BufferRenderer::_render_batch (src/renderers/buffer_renderer.hpp:
 *     151-250), with a run-time settle count.
 * Deviation (documented): a NaN final point is not binned, where the
 * reference converts NaN to size_t (undefined behaviour,
 * buffer_renderer.hpp:202); an index at or past the last cell is dropped and
 * counted, where the reference would write out of bounds.
 *
 * Stream model: stream s of seed S is seeded by key(S,s) = S + fmix64(s);
 * trajectory j of a job (length L, last one shorter) runs on stream
 * j mod STREAMS, in increasing j.
 */
#define _GNU_SOURCE
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "chaos_oracle.h"

/* ------------------------------------------------------------ ISAAC64/16 */
#define IS_N 16u

typedef struct {
    uint64_t rsl[IS_N];
    uint64_t mem[IS_N];
    uint64_t a, b, c;
    uint32_t cnt;
} isaac_t;

#define IS_MIX(a,b,c,d,e,f,g,h) do { \
    a -= e; f ^= h >>  9; h += a; \
    b -= f; g ^= a <<  9; a += b; \
    c -= g; h ^= b >> 23; b += c; \
    d -= h; a ^= c << 15; c += d; \
    e -= a; b ^= d >> 14; d += e; \
    f -= b; c ^= e << 20; e += f; \
    g -= c; d ^= f >> 17; f += g; \
    h -= d; e ^= g << 14; g += h; } while (0)

static void isaac_gen(isaac_t *s)
{
    uint64_t a = s->a, b = s->b + (++s->c);
    uint64_t *mm = s->mem;
    for (uint32_t i = 0; i < IS_N; ++i) {
        uint64_t x = mm[i];
        uint64_t mixv;
        switch (i & 3u) {
        case 0: mixv = ~(a ^ (a << 21)); break;
        case 1: mixv = a ^ (a >> 5); break;
        case 2: mixv = a ^ (a << 12); break;
        default: mixv = a ^ (a >> 33); break;
        }
        a = mixv + mm[(i + IS_N / 2) & (IS_N - 1)];
        uint64_t y = mm[(x >> 3) & (IS_N - 1)] + a + b;
        mm[i] = y;
        b = mm[(y >> (3 + 4)) & (IS_N - 1)] + x;
        s->rsl[i] = b;
    }
    s->a = a;
    s->b = b;
}

void oracle_isaac_seed(void *state, uint64_t key)
{
    isaac_t *s = (isaac_t *)state;
    uint64_t a, b, c, d, e, f, g, h;
    a = b = c = d = e = f = g = h = 0x9e3779b97f4a7c13ULL;
    for (int i = 0; i < 4; ++i)
        IS_MIX(a, b, c, d, e, f, g, h);
    for (uint32_t i = 0; i < IS_N; i += 8) {
        IS_MIX(a, b, c, d, e, f, g, h);
        s->mem[i + 0] = a; s->mem[i + 1] = b; s->mem[i + 2] = c;
        s->mem[i + 3] = d; s->mem[i + 4] = e; s->mem[i + 5] = f;
        s->mem[i + 6] = g; s->mem[i + 7] = h;
    }
    memset(s->rsl, 0, sizeof s->rsl);
    s->a = key;
    s->b = ~key;
    s->c = key ^ 11713835213681433683ULL;
    isaac_gen(s);
    s->cnt = IS_N;
}

static inline uint64_t isaac_next(isaac_t *s)
{
    if (s->cnt-- == 0) {
        isaac_gen(s);
        s->cnt = IS_N - 1;
    }
    return s->rsl[s->cnt];
}

size_t oracle_isaac_state_bytes(void) { return sizeof(isaac_t); }

void oracle_isaac_words(uint64_t key, uint64_t n, uint64_t *out)
{
    isaac_t s;
    oracle_isaac_seed(&s, key);
    for (uint64_t i = 0; i < n; ++i)
        out[i] = isaac_next(&s);
}

uint64_t oracle_fmix64(uint64_t k)
{
    k ^= k >> 33;
    k *= 0xff51afd7ed558ccdULL;
    k ^= k >> 33;
    k *= 0xc4ceb9fe1a85ec53ULL;
    k ^= k >> 33;
    return k;
}

uint64_t oracle_stream_key(uint64_t seed, uint64_t stream)
{
    return seed + oracle_fmix64(stream);
}

static inline double rand_num(isaac_t *s)
{
    return (double)(isaac_next(s) >> 11) / 9007199254740992.0;
}

static inline int rand_bool(isaac_t *s)
{
    return (int)(isaac_next(s) & 1u);
}

/* ------------------------------------------------------------ variations */
#define EPS 1e-20
#define BAD_THRESHOLD 1e20

/* sum of squares in coordinate order: Point::normsum<2> (point.hpp:300-307) */
static inline double nsq(const double *t, int n)
{
    double r = t[0] * t[0];
    for (int i = 1; i < n; ++i)
        r += t[i] * t[i];
    return r;
}

/* Point::norm<2> (point.hpp:270-290): |x| in 1-D, else sqrt(normsum<2>) */
static inline double n2(const double *t, int n)
{
    if (n == 1)
        return fabs(t[0]);
    return sqrt(nsq(t, n));
}

/*
 * One variation V(t) into out[0..dims).  2-D variations act on
 * (t[axis_x], t[axis_y]) and zero the other coordinates when dims > 2
 * (VariationFrom2D, variations.hpp:63-107).
 */
static void or_variation(const or_var *v, int dims, const double *t,
    double *out, isaac_t *rng)
{
    double x, y, r, a, s, c;
    int ax = v->axis_x, ay = v->axis_y;
    double o2[2] = {0.0, 0.0};
    int is2d = 0;
    switch (v->type) {
    case OR_V_LINEAR: /* variations.hpp:169-177 */
        for (int i = 0; i < dims; ++i)
            out[i] = t[i];
        return;
    case OR_V_SINUSOIDAL: /* variations.hpp:183-191 */
        for (int i = 0; i < dims; ++i)
            out[i] = sin(t[i]);
        return;
    case OR_V_SPHERICAL: /* variations.hpp:197-208 */
        r = 1.0 / (nsq(t, dims) + EPS);
        for (int i = 0; i < dims; ++i)
            out[i] = t[i] * r;
        return;
    case OR_V_SWIRL: /* variations.hpp:509-522 */
        x = t[ax]; y = t[ay];
        r = x * x + y * y;
        sincos(r, &s, &c);
        o2[0] = x * s - y * c;
        o2[1] = x * c + y * s;
        is2d = 1;
        break;
    case OR_V_HORSESHOE: /* variations.hpp:527-540 */
        x = t[ax]; y = t[ay];
        r = 1.0 / (sqrt(x * x + y * y) + EPS);
        o2[0] = ((x - y) * (x + y)) * r;
        o2[1] = (2.0 * x * y) * r;
        is2d = 1;
        break;
    case OR_V_POLAR: /* variations.hpp:545-555 */
        x = t[ax]; y = t[ay];
        a = atan2(y, x);
        r = sqrt(x * x + y * y);
        o2[0] = a * M_1_PI;
        o2[1] = r - 1.0;
        is2d = 1;
        break;
    case OR_V_JULIA: /* variations.hpp:807-819 */
        x = t[ax]; y = t[ay];
        a = 0.5 * atan2(y, x) + (double)rand_bool(rng) * M_PI;
        sincos(a, &s, &c);
        r = sqrt(x * x + y * y);
        o2[0] = c * r;
        o2[1] = s * r;
        is2d = 1;
        break;
    default:
        for (int i = 0; i < dims; ++i)
            out[i] = NAN;
        return;
    }
    if (is2d) {
        if (dims == 2) {
            out[0] = o2[0];
            out[1] = o2[1];
        } else {
            for (int i = 0; i < dims; ++i)
                out[i] = 0.0;
            out[ax] = o2[0];
            out[ay] = o2[1];
        }
    }
}

/* Affine::apply_to: ret = b; ret[i] += (0 + A[i][0]*x[0] + ...) */
static inline void affine(const double *A, const double *b, int n,
    const double *x, double *out)
{
    for (int i = 0; i < n; ++i) {
        double d = 0.0;
        for (int j = 0; j < n; ++j)
            d += A[i * n + j] * x[j];
        out[i] = b[i] + d;
    }
}

/* XForm::applyIteration (xform.hpp:211-227) */
static void apply_xform(const or_flame *f, const or_xform *xf,
    const double *p, double *out, isaac_t *rng)
{
    const int n = f->dims;
    double t[OR_MAXD], v[OR_MAXD], tmp[OR_MAXD];
    if (n < 3 || xf->has_pre)
        affine(xf->pre_A, xf->pre_b, n, p, t);
    else
        for (int i = 0; i < n; ++i)
            t[i] = p[i];
    for (int i = 0; i < n; ++i)
        v[i] = 0.0;
    for (int k = 0; k < xf->var_count; ++k) {
        const or_var *var = &f->vars[xf->var_begin + k];
        or_variation(var, n, t, tmp, rng);
        for (int i = 0; i < n; ++i)
            v[i] += tmp[i] * var->weight;
    }
    if (n < 3 || xf->has_post)
        affine(xf->post_A, xf->post_b, n, v, out);
    else
        for (int i = 0; i < n; ++i)
            out[i] = v[i];
}

/* Flame::getRandomXForm: first i with xfcw[i] >= r */
static inline int pick_xform(const or_flame *f, isaac_t *rng)
{
    double r = rand_num(rng);
    int i = 0;
    while (f->xfcw[i] < r)
        ++i;
    return i;
}

int oracle_pick_sequence(const or_flame *f, uint64_t key, uint64_t n,
    int32_t *out)
{
    isaac_t s;
    oracle_isaac_seed(&s, key);
    for (uint64_t i = 0; i < n; ++i)
        out[i] = pick_xform(f, &s);
    return 0;
}

int oracle_step(const or_flame *f, int xf_index, uint64_t key,
    uint64_t npts, const double *in, double *out)
{
    const or_xform *xf = xf_index < 0 ? &f->xf[f->nxf] : &f->xf[xf_index];
    if (xf_index < 0 && !f->has_final)
        return -1;
    if (xf_index >= f->nxf)
        return -1;
    for (uint64_t k = 0; k < npts; ++k) {
        isaac_t s;
        oracle_isaac_seed(&s, oracle_stream_key(key, k));
        apply_xform(f, xf, in + k * f->dims, out + k * f->dims, &s);
    }
    return 0;
}

/* ------------------------------------------------------------ trajectory */
typedef struct {
    const or_flame *f;
    uint64_t settle;
    double p[OR_MAXD], pf[OR_MAXD];
    double c[OR_MAXC], cf[OR_MAXC];
} iter_t;

static void iter_init(iter_t *it, isaac_t *rng)
{
    const or_flame *f = it->f;
    for (int i = 0; i < f->dims; ++i)
        it->p[i] = 2.0 * rand_num(rng) - 1.0;
    for (uint64_t k = 0; k < it->settle; ++k) {
        double q[OR_MAXD];
        apply_xform(f, &f->xf[pick_xform(f, rng)], it->p, q, rng);
        memcpy(it->p, q, sizeof q);
    }
    for (int i = 0; i < f->color_dims; ++i)
        it->c[i] = rand_num(rng);
}

typedef struct {
    uint64_t s_iter, s_plot, bad, dropped;
    uint64_t *xf_dist;          /* xform_ids entries */
    double ext_lo[OR_MAXD], ext_hi[OR_MAXD];
} local_stats_t;

typedef struct {
    const or_flame *f;
    uint64_t seed, streams, samples, traj_len, settle, bad_limit;
    uint64_t *counts;
    double *colors;
    volatile uint64_t *bad_total;
    uint64_t s_begin, s_end;
    local_stats_t st;
    int stopped;
    double mult_d[OR_MAXD];
    uint64_t mult_i[OR_MAXD], cells;
} work_t;

/* one trajectory of `len` samples (BufferRenderer::_render_batch) */
static int render_batch(work_t *w, isaac_t *rng, uint64_t len)
{
    const or_flame *f = w->f;
    const int n = f->dims, r = f->color_dims;
    if (__atomic_load_n(w->bad_total, __ATOMIC_RELAXED) > w->bad_limit)
        return 0;
    iter_t it;
    it.f = f;
    it.settle = w->settle;
    iter_init(&it, rng);
    for (; len > 0; --len) {
        int xi = pick_xform(f, rng);
        const or_xform *xf = &f->xf[xi];
        double q[OR_MAXD];
        apply_xform(f, xf, it.p, q, rng);
        memcpy(it.p, q, sizeof q);
        if (r && xf->has_color) {
            const double s = xf->color_speed;
            for (int i = 0; i < r; ++i)
                it.c[i] = (1.0 - s) * it.c[i] + s * f->colors[xi * r + i];
        }
        if (f->has_final) {
            const or_xform *ff = &f->xf[f->nxf];
            apply_xform(f, ff, it.p, it.pf, rng);
            if (r) {
                if (ff->has_color) {
                    const double s = ff->color_speed;
                    for (int i = 0; i < r; ++i)
                        it.cf[i] = (1.0 - s) * it.c[i]
                            + s * f->colors[f->nxf * r + i];
                } else
                    for (int i = 0; i < r; ++i)
                        it.cf[i] = it.c[i];
            }
        } else {
            memcpy(it.pf, it.p, sizeof it.p);
            for (int i = 0; i < r; ++i)
                it.cf[i] = it.c[i];
        }
        ++w->st.s_iter;
        ++w->st.xf_dist[xf->id];
        int badv = 0;
        for (int i = 0; i < n; ++i)
            if (fabs(it.p[i]) > BAD_THRESHOLD || isnan(it.p[i]))
                badv = 1;
        if (badv) {
            ++w->st.bad;
            uint64_t tot = __atomic_add_fetch(w->bad_total, 1, __ATOMIC_RELAXED);
            if (tot > w->bad_limit)
                break;
            iter_init(&it, rng);
        }
        for (int i = 0; i < n; ++i) {
            if (it.p[i] < w->st.ext_lo[i]) w->st.ext_lo[i] = it.p[i];
            if (it.p[i] > w->st.ext_hi[i]) w->st.ext_hi[i] = it.p[i];
        }
        int inb = 1;
        for (int i = 0; i < n; ++i)
            if (isnan(it.pf[i]) || it.pf[i] < f->lo[i] || it.pf[i] > f->hi[i])
                inb = 0;
        if (!inb)
            continue;
        ++w->st.s_plot;
        uint64_t bi = (uint64_t)((it.pf[0] - f->lo[0]) * w->mult_d[0]);
        for (int i = 1; i < n; ++i)
            bi += (uint64_t)((it.pf[i] - f->lo[i]) * w->mult_d[i]) * w->mult_i[i];
        if (bi >= w->cells) {
            ++w->st.dropped;
            continue;
        }
        __atomic_add_fetch(&w->counts[bi], 1, __ATOMIC_RELAXED);
        for (int i = 0; i < r; ++i) {
            /* f64 add by CAS, as std::atomic<double>::fetch_add */
            double *dp = &w->colors[bi * r + i];
            uint64_t *up = (uint64_t *)dp;
            uint64_t oldu = __atomic_load_n(up, __ATOMIC_RELAXED), newu;
            do {
                double od, nd;
                memcpy(&od, &oldu, 8);
                nd = od + it.cf[i];
                memcpy(&newu, &nd, 8);
            } while (!__atomic_compare_exchange_n(up, &oldu, newu, 1,
                         __ATOMIC_RELAXED, __ATOMIC_RELAXED));
        }
    }
    return len == 0;
}

static void *render_worker(void *arg)
{
    work_t *w = (work_t *)arg;
    const uint64_t ntraj = (w->samples + w->traj_len - 1) / w->traj_len;
    for (uint64_t s = w->s_begin; s < w->s_end && !w->stopped; ++s) {
        isaac_t rng;
        oracle_isaac_seed(&rng, oracle_stream_key(w->seed, s));
        for (uint64_t t = s; t < ntraj; t += w->streams) {
            uint64_t len = w->samples - t * w->traj_len;
            if (len > w->traj_len)
                len = w->traj_len;
            if (!render_batch(w, &rng, len)) {
                w->stopped = 1;
                break;
            }
        }
    }
    return NULL;
}

void oracle_index_mults(const or_flame *f, double *mult_d, uint64_t *mult_i,
    uint64_t *cells)
{
    uint64_t c = 1;
    for (int i = 0; i < f->dims; ++i) {
        mult_d[i] = (double)f->size[i] / (f->hi[i] - f->lo[i]);
        mult_d[i] *= 1.0 - 1.0 / 4503599627370496.0; /* 1 - 2^-52 */
        mult_i[i] = c;
        c *= f->size[i];
    }
    *cells = c;
}

int oracle_render(const or_flame *f, uint64_t seed, uint64_t streams,
    uint64_t samples, uint64_t traj_len, uint64_t settle, uint64_t bad_limit,
    int threads, uint64_t *counts, double *colors, or_stats *out)
{
    if (f->dims < 1 || f->dims > OR_MAXD || f->color_dims > OR_MAXC
            || f->nxf < 1 || streams == 0 || traj_len == 0)
        return -1;
    if (threads < 1)
        threads = 1;
    const uint64_t ntraj = samples ? (samples + traj_len - 1) / traj_len : 0;
    uint64_t used = streams < ntraj ? streams : ntraj;
    if ((uint64_t)threads > used)
        threads = used ? (int)used : 1;
    volatile uint64_t bad_total = 0;
    work_t *ws = (work_t *)calloc((size_t)threads, sizeof(work_t));
    pthread_t *tids = (pthread_t *)calloc((size_t)threads, sizeof(pthread_t));
    for (int k = 0; k < threads; ++k) {
        work_t *w = &ws[k];
        w->f = f;
        w->seed = seed; w->streams = streams; w->samples = samples;
        w->traj_len = traj_len; w->settle = settle; w->bad_limit = bad_limit;
        w->counts = counts; w->colors = colors; w->bad_total = &bad_total;
        w->s_begin = used * (uint64_t)k / (uint64_t)threads;
        w->s_end = used * (uint64_t)(k + 1) / (uint64_t)threads;
        w->st.xf_dist = (uint64_t *)calloc((size_t)f->xform_ids + 1, 8);
        for (int i = 0; i < OR_MAXD; ++i) {
            w->st.ext_lo[i] = INFINITY;
            w->st.ext_hi[i] = -INFINITY;
        }
        oracle_index_mults(f, w->mult_d, w->mult_i, &w->cells);
    }
    if (threads == 1)
        render_worker(&ws[0]);
    else {
        for (int k = 0; k < threads; ++k)
            pthread_create(&tids[k], NULL, render_worker, &ws[k]);
        for (int k = 0; k < threads; ++k)
            pthread_join(tids[k], NULL);
    }
    memset(out, 0, sizeof *out);
    for (int i = 0; i < OR_MAXD; ++i) {
        out->ext_lo[i] = INFINITY;
        out->ext_hi[i] = -INFINITY;
    }
    int ok = 1;
    for (int k = 0; k < threads; ++k) {
        work_t *w = &ws[k];
        out->s_iter += w->st.s_iter;
        out->s_plot += w->st.s_plot;
        out->bad += w->st.bad;
        out->dropped += w->st.dropped;
        for (int i = 0; i < f->xform_ids && i < OR_MAXX; ++i)
            out->xf_dist[i] += w->st.xf_dist[i];
        for (int i = 0; i < f->dims; ++i) {
            if (w->st.ext_lo[i] < out->ext_lo[i]) out->ext_lo[i] = w->st.ext_lo[i];
            if (w->st.ext_hi[i] > out->ext_hi[i]) out->ext_hi[i] = w->st.ext_hi[i];
        }
        if (w->stopped)
            ok = 0;
        free(w->st.xf_dist);
    }
    out->ok = ok;
    free(ws);
    free(tids);
    return 0;
}

int oracle_trace(const or_flame *f, uint64_t key, uint64_t settle,
    uint64_t n, int32_t *ids, double *pts)
{
    isaac_t rng;
    oracle_isaac_seed(&rng, key);
    iter_t it;
    it.f = f;
    it.settle = settle;
    for (int i = 0; i < f->dims; ++i)
        it.p[i] = 2.0 * rand_num(&rng) - 1.0;
    for (uint64_t k = 0; k < settle; ++k) {
        double q[OR_MAXD];
        apply_xform(f, &f->xf[pick_xform(f, &rng)], it.p, q, &rng);
        memcpy(it.p, q, sizeof q);
    }
    for (uint64_t k = 0; k < n; ++k) {
        int xi = pick_xform(f, &rng);
        double q[OR_MAXD];
        apply_xform(f, &f->xf[xi], it.p, q, &rng);
        memcpy(it.p, q, sizeof q);
        ids[k] = (int32_t)f->xf[xi].id;
        for (int i = 0; i < f->dims; ++i)
            pts[k * f->dims + i] = it.p[i];
    }
    return 0;
}

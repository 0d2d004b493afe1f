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

static inline double rand_gauss(isaac_t *s)
{
    /* FlameRNG::randGaussianPair (flame_rng.hpp:115-140), first value */
    double u1 = rand_num(s);
    double u2 = (2.0 * M_PI) * rand_num(s);
    double r = sqrt(-2.0 * log(u1));
    double sn, cs;
    sincos(u2, &sn, &cs);
    return r * cs;
}

/* FlameRNG::randGaussianPair (flame_rng.hpp:115-140), both values */
static inline void rand_gauss_pair(isaac_t *s, double *z1, double *z2)
{
    double u1 = rand_num(s);
    double u2 = (2.0 * M_PI) * rand_num(s);
    double r = sqrt(-2.0 * log(u1));
    double sn, cs;
    sincos(u2, &sn, &cs);
    *z1 = r * cs;
    *z2 = r * sn;
}

/* FlameRNG::randDirection<dims> (flame_rng.hpp:171-217); above 3 dims a
   vector of gaussian pairs (the last one's second value unused for odd
   dims) divided by its norm, Point / k being multiplication by 1 / k */
static inline void rand_dir(isaac_t *s, int dims, double *d)
{
    if (dims > 3) {
        double unused, n2 = 0.0, k;
        int i;
        for (i = 0; i + 1 < dims; i += 2)
            rand_gauss_pair(s, &d[i], &d[i + 1]);
        if (dims % 2)
            rand_gauss_pair(s, &d[dims - 1], &unused);
        for (i = 0; i < dims; ++i)
            n2 += d[i] * d[i];
        k = 1.0 / sqrt(n2);
        for (i = 0; i < dims; ++i)
            d[i] *= k;
        return;
    }
    if (dims == 1) {
        d[0] = copysign(1.0, rand_num(s) - 0.5);
    } else if (dims == 2) {
        double a = (2.0 * M_PI) * rand_num(s);
        double sa, ca;
        sincos(a, &sa, &ca);
        d[0] = ca;
        d[1] = sa;
    } else {
        double u = 2.0 * rand_num(s) - 1.0;
        double t = (2.0 * M_PI) * rand_num(s);
        double r = sqrt(1.0 - u * u);
        double st, ct;
        sincos(t, &st, &ct);
        d[0] = r * ct;
        d[1] = r * st;
        d[2] = u;
    }
}

/* RNG words one call of each variation draws (fixed per variation) */
int oracle_variation_words(int type, int dims)
{
    /* randDirection<dims> draws: 1 (dims 1, 2), 2 (dims 3), 2 per gaussian
       pair above 3 dims */
    int dw = dims == 3 ? 2 : (dims > 3 ? 2 * ((dims + 1) / 2) : 1);
    switch (type) {
    case OR_V_NOISE: case OR_V_BLUR: return 1 + dw;
    case OR_V_GAUSSIAN_BLUR: case OR_V_PRE_BLUR: return 2 + dw;
    case OR_V_SQUARE_NOISE: return dims;
    case OR_V_JULIA: case OR_V_JULIAN: case OR_V_ARCH: case OR_V_RAYS:
    case OR_V_BLADE: case OR_V_TWINTRIAN: case OR_V_WEDGE_JULIA:
    case OR_V_SUPERSHAPE: case OR_V_FLOWER: case OR_V_CONIC:
    case OR_V_BOARDERS: case OR_V_CPOW: return 1;
    case OR_V_JULIASCOPE: case OR_V_RADIAL_BLUR: case OR_V_PARABOLA: return 2;
    case OR_V_PIE: return 3;
    default: return 0;
    }
}

/* Point::normsum(p) (point.hpp:325-331) */
static inline double normsum_p(const double *t, int n, double p)
{
    double r = pow(fabs(t[0]), p);
    for (int i = 1; i < n; ++i)
        r += pow(fabs(t[i]), p);
    return r;
}

#define EPS 1e-20
#define BAD_THRESHOLD 1e20

/*
 * One variation V(t) into out[0..dims).  2-D variations act on
 * (t[axis_x], t[axis_y]) and zero the other coordinates when dims > 2
 * (VariationFrom2D, variations.hpp:63-107).  Each case restates the class
 * of src/variations/variations.hpp at the line given, in the same operation
 * order.  Point / k is computed as multiplication by (1/k), as
 * Point::operator/= does (point.hpp:127-131).
 */
static void or_variation(const or_var *v, int dims, const double *t,
    double *out, isaac_t *rng)
{
    const double *P = v->params;
    double x, y, r, a, s, c, X = 0.0, Y = 0.0, d;
    int i;
    if (v->type < OR_FIRST_2D) {
        switch (v->type) {
        case OR_V_LINEAR: /* 169-177 */
            for (i = 0; i < dims; ++i) out[i] = t[i];
            return;
        case OR_V_SINUSOIDAL: /* 183-191 */
            for (i = 0; i < dims; ++i) out[i] = sin(t[i]);
            return;
        case OR_V_SPHERICAL: /* 197-208 */
            r = 1.0 / (nsq(t, dims) + EPS);
            for (i = 0; i < dims; ++i) out[i] = t[i] * r;
            return;
        case OR_V_BENT: /* 216-240: p = neg[dims], pos[dims] */
            for (i = 0; i < dims; ++i)
                out[i] = t[i] < 0.0 ? t[i] * P[i] : t[i] * P[dims + i];
            return;
        case OR_V_RECTANGLES: /* 245-270 */
            for (i = 0; i < dims; ++i)
                out[i] = P[i] == 0.0 ? t[i]
                    : (2.0 * floor(t[i] / P[i]) + 1.0) * P[i] - t[i];
            return;
        case OR_V_FISHEYE: /* 275-292: p = addval */
            r = 1.0 / (n2(t, dims) + P[0]);
            for (i = 0; i < dims; ++i) out[i] = t[i] * r;
            return;
        case OR_V_BUBBLE: /* 297-314 */
            r = 1.0 / (nsq(t, dims) + P[0]);
            for (i = 0; i < dims; ++i) out[i] = t[i] * r;
            return;
        case OR_V_NOISE: { /* 319-330 */
            double dir[OR_MAXD];
            r = rand_num(rng);
            rand_dir(rng, dims, dir);
            for (i = 0; i < dims; ++i) out[i] = (t[i] * dir[i]) * r;
            return;
        }
        case OR_V_BLUR: { /* 335-347 */
            double dir[OR_MAXD];
            r = rand_num(rng);
            rand_dir(rng, dims, dir);
            for (i = 0; i < dims; ++i) out[i] = dir[i] * r;
            return;
        }
        case OR_V_GAUSSIAN_BLUR: /* 352-364 */
        case OR_V_PRE_BLUR: { /* 434-446 */
            double dir[OR_MAXD];
            r = rand_gauss(rng);
            rand_dir(rng, dims, dir);
            for (i = 0; i < dims; ++i) out[i] = dir[i] * r;
            return;
        }
        case OR_V_SQUARE_NOISE: /* 369-378, randPoint2 */
            for (i = 0; i < dims; ++i) out[i] = rand_num(rng) - 0.5;
            return;
        case OR_V_SEPARATION: /* 383-405: p = sep^2[dims], inside[dims] */
            for (i = 0; i < dims; ++i) {
                s = copysign(1.0, t[i]);
                out[i] = s * (sqrt(t[i] * t[i] + P[i]) - s * P[dims + i]);
            }
            return;
        case OR_V_SPLITS: /* 410-429 */
            for (i = 0; i < dims; ++i) {
                s = copysign(1.0, t[i]);
                out[i] = t[i] + s * P[i];
            }
            return;
        case OR_V_MODULUS: /* 451-471: p = 2*params, 1/(2*params) */
            for (i = 0; i < dims; ++i)
                out[i] = t[i] - P[i] * floor(t[i] * P[dims + i] + 0.5);
            return;
        case OR_V_CELLN: /* 476-505: p = sizes, 1/sizes */
            for (i = 0; i < dims; ++i) {
                double fx = floor(t[i] * P[dims + i]);
                double dx = t[i] - fx * P[i];
                double xs = copysign(2.0, fx);
                double x2 = fx * xs;
                x2 -= (double)(fx < 0);
                out[i] = dx + x2 * P[i];
            }
            return;
        case OR_V_SPHERICAL_P: /* 2312-2328 */
            r = 1.0 / (normsum_p(t, dims, P[0]) + EPS);
            for (i = 0; i < dims; ++i) out[i] = t[i] * r;
            return;
        case OR_V_UNIT_SPHERE: /* 2333-2342 */
            r = 1.0 / (n2(t, dims) + EPS);
            for (i = 0; i < dims; ++i) out[i] = t[i] * r;
            return;
        case OR_V_UNIT_SPHERE_P: /* 2347-2363: norm(p) = pow(normsum, 1/p) */
            r = 1.0 / (pow(normsum_p(t, dims, P[0]), 1.0 / P[0]) + EPS);
            for (i = 0; i < dims; ++i) out[i] = t[i] * r;
            return;
        case OR_V_UNIT_CUBE: { /* 2368-2376: norm<0> */
            double m = fabs(t[0]);
            if (dims > 1)
                for (i = 1; i < dims; ++i) {
                    double q = fabs(t[i]);
                    m = (m < q) ? q : m;
                }
            r = 1.0 / (m + EPS);
            for (i = 0; i < dims; ++i) out[i] = t[i] * r;
            return;
        }
        default:
            for (i = 0; i < dims; ++i) out[i] = NAN;
            return;
        }
    }
    x = t[v->axis_x];
    y = t[v->axis_y];
#define R2SQ (x * x + y * y)
#define R2 sqrt(x * x + y * y)
#define ANG atan2(y, x)
    switch (v->type) {
    case OR_V_SWIRL: /* 509-522 */
        r = R2SQ; sincos(r, &s, &c);
        X = x * s - y * c; Y = x * c + y * s; break;
    case OR_V_HORSESHOE: /* 527-540 */
        r = 1.0 / (R2 + EPS);
        X = ((x - y) * (x + y)) * r; Y = (2.0 * x * y) * r; break;
    case OR_V_POLAR: /* 545-555 */
        a = ANG; r = R2; X = a * M_1_PI; Y = r - 1.0; break;
    case OR_V_POLAR2: /* 561-570 */
        X = ANG; Y = log(R2SQ); break;
    case OR_V_HANDKERCHIEF: /* 575-585 */
        a = ANG; r = R2; X = sin(a + r) * r; Y = cos(a - r) * r; break;
    case OR_V_HEART: /* 590-602 */
        a = ANG; r = R2; sincos(r * a, &s, &c); X = s * r; Y = (-c) * r; break;
    case OR_V_DISC: /* 607-619 */
        a = ANG; r = R2; sincos(M_PI * r, &s, &c); X = s * a; Y = c * a; break;
    case OR_V_DISC2: /* 624-655: p = rotpi, cosadd, sinadd */
        d = P[0] * (x + y); sincos(d, &s, &c); a = ANG;
        X = (c + P[1]) * a; Y = (s + P[2]) * a; break;
    case OR_V_WAVES: /* 660-680: p = xf, xs, yf, ys */
        X = x + P[1] * sin(y * P[0]); Y = y + P[3] * sin(x * P[2]); break;
    case OR_V_FAN: { /* 685-709: p = dx, dy */
        double dx2 = P[0] * 0.5;
        a = ANG;
        double m = copysign(1.0, dx2 - fmod(a + P[1], P[0]));
        a += m * dx2;
        sincos(a, &s, &c);
        r = R2;
        X = c * r; Y = s * r; break;
    }
    case OR_V_RINGS: /* 714-733: p = dx */
        r = R2; s = y / r; c = x / r;
        r = fmod(r + P[0], 2.0 * P[0]) - P[0] + r * (1.0 - P[0]);
        X = c * r; Y = s * r; break;
    case OR_V_SPIRAL: { /* 738-752 */
        double sa, ca, sr, cr;
        r = R2; sa = y / r; ca = x / r;
        sincos(r, &sr, &cr);
        double r1 = 1.0 / (r + EPS);
        X = (ca + sr) * r1; Y = (sa - cr) * r1; break;
    }
    case OR_V_HYPERBOLIC: /* 757-767 */
        r = R2; s = y / r; c = x / r;
        X = s / (r + EPS); Y = c * r; break;
    case OR_V_DIAMOND: { /* 772-784 */
        double sr, cr;
        r = R2; s = y / r; c = x / r;
        sincos(r, &sr, &cr);
        X = s * cr; Y = c * sr; break;
    }
    case OR_V_EX: { /* 789-803 */
        a = ANG; r = R2;
        double n0 = sin(a + r), n1 = cos(a - r);
        double m0 = n0 * n0 * n0 * r, m1 = n1 * n1 * n1 * r;
        X = m0 + m1; Y = m0 - m1; break;
    }
    case OR_V_JULIA: /* 807-819 */
        a = 0.5 * atan2(y, x) + (double)rand_bool(rng) * M_PI;
        sincos(a, &s, &c);
        r = R2;
        X = c * r; Y = s * r; break;
    case OR_V_EXPONENTIAL: /* 825-838 */
        d = exp(x - 1.0); sincos(M_PI * y, &s, &c);
        X = c * d; Y = s * d; break;
    case OR_V_POWER: /* 843-853 */
        r = R2; s = y / r; c = x / r; d = pow(r, s);
        X = c * d; Y = s * d; break;
    case OR_V_COSINE: /* 858-870 */
        sincos(x * M_PI, &s, &c);
        X = c * cosh(y); Y = (-s) * sinh(y); break;
    case OR_V_BLOB: /* 875-896: p = mid, amp, waves */
        r = R2; s = y / r; c = x / r; a = ANG;
        r *= P[0] + P[1] * sin(P[2] * a);
        X = c * r; Y = s * r; break;
    case OR_V_PDJ: /* 901-925: p = a, b, c, d */
        X = sin(P[0] * y) - cos(P[1] * x); Y = sin(P[2] * x) - cos(P[3] * y); break;
    case OR_V_CYLINDER: /* 930-938 */
        X = sin(x); Y = y; break;
    case OR_V_PERSPECTIVE: /* 943-962: p = dist, vsin, vfcos */
        d = 1.0 / (P[0] - y * P[1]);
        X = (P[0] * x) * d; Y = (P[2] * y) * d; break;
    case OR_V_JULIAN: { /* 967-989: p = abspower, invpower, cn */
        int32_t tt = (int32_t)trunc(P[0] * rand_num(rng));
        a = (atan2(y, x) + (2.0 * M_PI) * tt) * P[1];
        r = pow(R2SQ, P[2]);
        sincos(a, &s, &c);
        X = c * r; Y = s * r; break;
    }
    case OR_V_JULIASCOPE: { /* 994-1018 */
        int32_t tt = (int32_t)trunc(P[0] * rand_num(rng));
        double dir = copysign(1.0, rand_num(rng) - 0.5);
        a = ((2.0 * M_PI) * tt + dir * atan2(y, x)) * P[1];
        r = pow(R2SQ, P[2]);
        sincos(a, &s, &c);
        X = c * r; Y = s * r; break;
    }
    case OR_V_RADIAL_BLUR: { /* 1023-1045: p = spin, zoom, flam3weight */
        double g = P[2] * rand_gauss(rng);
        double ra = R2;
        a = atan2(y, x) + P[0] * g;
        sincos(a, &s, &c);
        double rz = P[1] * g - 1.0;
        X = c * ra + x * rz; Y = s * ra + y * rz; break;
    }
    case OR_V_PIE: { /* 1050-1072: p = slices, rotation, thickness, invslices2pi */
        int32_t sl = (int32_t)(rand_num(rng) * P[0] + 0.5);
        a = P[1] + (sl + rand_num(rng) * P[2]) * P[3];
        r = rand_num(rng);
        sincos(a, &s, &c);
        X = c * r; Y = s * r; break;
    }
    case OR_V_NGON: { /* 1077-1102: p = powerval, angle, corners, circle, invangle */
        r = pow(R2SQ, P[0]);
        double theta = atan2(y, x);
        double phi = theta - P[1] * floor(theta * P[4]);
        phi -= (phi > P[1] * 0.5 ? 1.0 : 0.0) * P[1];
        double amp = P[2] * (1.0 / (cos(phi) + EPS) - 1.0) + P[3];
        amp /= r + EPS;
        X = x * amp; Y = y * amp; break;
    }
    case OR_V_CURL: { /* 1107-1129: p = c1, c2 */
        double re = 1.0 + P[0] * x + P[1] * (x * x - y * y);
        double im = P[0] * y + 2.0 * P[1] * x * y;
        r = 1.0 / (re * re + im * im + EPS);
        X = (x * re + y * im) * r; Y = (y * re - x * im) * r; break;
    }
    case OR_V_ARCH: /* 1134-1151: p = flam3weight */
        a = P[0] * rand_num(rng) * M_PI;
        sincos(a, &s, &c);
        X = s; Y = s * s / c; break;
    case OR_V_TANGENT: /* 1156-1166 */
        X = sin(x) / cos(y); Y = tan(y); break;
    case OR_V_RAYS: /* 1172-1191 */
        a = P[0] * rand_num(rng) * M_PI;
        r = P[0] / (R2SQ + EPS);
        d = tan(a) * r;
        X = cos(x) * d; Y = sin(y) * d; break;
    case OR_V_BLADE: { /* 1196-1213 */
        double sr, cr;
        r = rand_num(rng) * P[0] * R2;
        sincos(r, &sr, &cr);
        X = (cr + sr) * x; Y = (cr - sr) * x; break;
    }
    case OR_V_SECANT: { /* 1218-1235 */
        double cr = cos(P[0] * R2);
        double icr = 1.0 / cr;
        double sg = copysign(1.0, -cr);
        X = x; Y = icr + sg; break;
    }
    case OR_V_TWINTRIAN: { /* 1240-1260 */
        double sr, cr;
        r = rand_num(rng) * P[0] * R2;
        sincos(r, &sr, &cr);
        double diff = log10(sr * sr) + cr;
        if (fabs(diff) > BAD_THRESHOLD || isnan(diff))
            diff = -30.0;
        X = diff * x; Y = (diff - sr * M_PI) * x; break;
    }
    case OR_V_CROSS: /* 1265-1277 */
        s = x * x - y * y;
        r = sqrt(1.0 / (s * s + EPS));
        X = x * r; Y = y * r; break;
    case OR_V_EXP: /* 1282-1295 */
        d = exp(x); sincos(y, &s, &c);
        X = c * d; Y = s * d; break;
    case OR_V_LOG: /* 1300-1308 */
        X = log(R2SQ); Y = atan2(y, x); break;
    case OR_V_SIN: /* 1313-1327 */
        sincos(x, &s, &c);
        X = s * cosh(y); Y = c * sinh(y); break;
    case OR_V_COS: /* 1332-1346 */
        sincos(x, &s, &c);
        { double ch = cosh(y), sh = sinh(y); X = c * ch; Y = (-s) * sh; }
        break;
    case OR_V_TAN: { /* 1351-1366 */
        sincos(2.0 * x, &s, &c);
        double sh = sinh(2.0 * y), ch = cosh(2.0 * y);
        d = 1.0 / (c + ch);
        X = s * d; Y = sh * d; break;
    }
    case OR_V_SEC: { /* 1371-1386 */
        sincos(x, &s, &c);
        double sh = sinh(y), ch = cosh(y);
        d = 1.0 / (cos(2.0 * x) + cosh(2.0 * y));
        X = (c * ch) * d; Y = (s * sh) * d; break;
    }
    case OR_V_CSC: { /* 1391-1406 */
        sincos(x, &s, &c);
        double sh = sinh(y), ch = cosh(y);
        d = 1.0 / (cosh(2.0 * y) - cos(2.0 * x));
        X = (s * ch) * d; Y = ((-c) * sh) * d; break;
    }
    case OR_V_COT: { /* 1411-1426 */
        sincos(2.0 * x, &s, &c);
        double sh = sinh(2.0 * y), ch = cosh(2.0 * y);
        d = 1.0 / (ch - c);
        X = s * d; Y = (-sh) * d; break;
    }
    case OR_V_SINH: { /* 1431-1445 */
        sincos(y, &s, &c);
        double sh = sinh(x), ch = cosh(x);
        X = sh * c; Y = ch * s; break;
    }
    case OR_V_COSH: { /* 1450-1464 */
        sincos(y, &s, &c);
        double sh = sinh(x), ch = cosh(x);
        X = ch * c; Y = sh * s; break;
    }
    case OR_V_TANH: { /* 1469-1484 */
        sincos(2.0 * y, &s, &c);
        double sh = sinh(2.0 * x), ch = cosh(2.0 * x);
        d = 1.0 / (c + ch);
        X = sh * d; Y = s * d; break;
    }
    case OR_V_SECH: { /* 1489-1504 */
        sincos(y, &s, &c);
        double sh = sinh(x), ch = cosh(x);
        d = 1.0 / (cos(2.0 * y) + cosh(2.0 * x));
        X = (c * ch) * d; Y = ((-s) * sh) * d; break;
    }
    case OR_V_CSCH: { /* 1509-1524 */
        sincos(y, &s, &c);
        double sh = sinh(x), ch = cosh(x);
        d = 1.0 / (cosh(2.0 * x) - cos(2.0 * y));
        X = (sh * c) * d; Y = ((-ch) * s) * d; break;
    }
    case OR_V_COTH: { /* 1529-1544 */
        sincos(2.0 * y, &s, &c);
        double sh = sinh(2.0 * x), ch = cosh(2.0 * x);
        d = 1.0 / (ch - c);
        X = sh * d; Y = s * d; break;
    }
    case OR_V_AUGER: { /* 1549-1571: p = freq, weight, scale/2, sym */
        double ss = sin(P[0] * x), tt = sin(P[0] * y);
        double dy = y + P[1] * (P[2] + fabs(y)) * ss;
        double dx = x + P[1] * (P[2] + fabs(x)) * tt;
        X = x + P[3] * (dx - x); Y = dy; break;
    }
    case OR_V_FLUX: { /* 1576-1600: p = 2 + spread, weight */
        double xpw = x + P[1], xmw = x - P[1], y2 = y * y;
        double avgr = P[0] * sqrt(sqrt(y2 + xpw * xpw) / sqrt(y2 + xmw * xmw));
        double avga = (atan2(y, xmw) - atan2(y, xpw)) * 0.5;
        /* sincosg(avga, c, s) stores the sine in c (variations.hpp:1597) */
        sincos(avga, &c, &s);
        X = c * avgr; Y = s * avgr; break;
    }
    case OR_V_MOBIUS: { /* 1605-1630: p = a0 a1 b0 b1 c0 c1 d0 d1 */
        double re_u = P[0] * x - P[1] * y + P[2];
        double im_u = P[0] * y + P[1] * x + P[3];
        double re_v = P[4] * x - P[5] * y + P[6];
        double im_v = P[4] * y + P[5] * x + P[7];
        double rad = 1.0 / (re_v * re_v + im_v * im_v + EPS);
        X = (re_u * re_v + im_u * im_v) * rad;
        Y = (im_u * re_v - re_u * im_v) * rad; break;
    }
    case OR_V_SCRY: { /* 1635-1650 */
        double tt = R2SQ;
        r = 1.0 / (sqrt(tt) * (tt + 1.0 / (P[0] + EPS)));
        X = x * r; Y = y * r; break;
    }
    case OR_V_SPLIT: { /* 1655-1673: p = xsize*pi, ysize*pi */
        double xs = copysign(1.0, cos(x * P[0]));
        double ys = copysign(1.0, cos(y * P[1]));
        X = x * ys; Y = y * xs; break;
    }
    case OR_V_STRIPES: { /* 1678-1696: p = 1 - space, warp */
        double rx = floor(x + 0.5), ox = x - rx;
        X = ox * P[0] + rx; Y = y + ox * ox * P[1]; break;
    }
    case OR_V_WEDGE: { /* 1701-1724: p = swirl, count, angle, hole, cf */
        r = R2;
        a = atan2(y, x) + P[0] * r;
        double cc = floor((P[1] * a + M_PI) * (M_1_PI * 0.5));
        a = a * P[4] + cc * P[2];
        sincos(a, &s, &c);
        X = c * (r + P[3]); Y = s * (r + P[3]); break;
    }
    case OR_V_WEDGE_JULIA: { /* 1729-1756: p = angle, count, invpower, cn, abspower, cf */
        r = pow(R2SQ, P[3]);
        int32_t tr = (int32_t)(P[4] * rand_num(rng));
        a = (atan2(y, x) + (2.0 * M_PI) * tr) * P[2];
        double cc = floor((P[1] * a + M_PI) * (M_1_PI * 0.5));
        a = a * P[5] + cc * P[0];
        sincos(a, &s, &c);
        X = c * r; Y = s * r; break;
    }
    case OR_V_WEDGE_SPH: { /* 1761-1785: p = angle, count, swirl, hole, cf */
        r = 1.0 / (R2 + EPS);
        a = atan2(y, x) + P[2] * r;
        double cc = floor((P[1] * a + M_PI) * (M_1_PI * 0.5));
        a = a * P[4] + cc * P[0];
        sincos(a, &s, &c);
        X = c * (r + P[3]); Y = s * (r + P[3]); break;
    }
    case OR_V_WHORL: /* 1790-1810: p = inside, outside, weight */
        r = R2;
        a = atan2(y, x);
        a += (r >= P[2] ? P[1] : P[0]) / (P[2] - r);
        sincos(a, &s, &c);
        X = c * r; Y = s * r; break;
    case OR_V_SUPERSHAPE: { /* 1815-1842: p = m/4, -1/n1, n2, n3, rnd, holes */
        double theta = P[0] * atan2(y, x) + M_PI_4;
        double st, ct;
        sincos(theta, &st, &ct);
        double t1 = pow(fabs(ct), P[2]), t2 = pow(fabs(st), P[3]);
        double tr = R2;
        r = (P[4] * rand_num(rng) + (1.0 - P[4]) * tr) - P[5];
        r *= pow(t1 + t2, P[1]) / tr;
        X = x * r; Y = y * r; break;
    }
    case OR_V_FLOWER: /* 1847-1864: p = petals, holes */
        r = (rand_num(rng) - P[1]) * cos(P[0] * atan2(y, x));
        r /= R2 + EPS;
        X = x * r; Y = y * r; break;
    case OR_V_CONIC: { /* 1869-1886: p = eccen, holes */
        double tr = R2;
        double ct = x / (tr + EPS);
        r = (rand_num(rng) - P[1]) * P[0] / (tr + tr * P[0] * ct);
        X = x * r; Y = y * r; break;
    }
    case OR_V_PARABOLA: { /* 1891-1909: p = height, width */
        double sr, cr;
        sincos(R2, &sr, &cr);
        X = P[0] * sr * sr * rand_num(rng);
        Y = P[1] * cr * rand_num(rng); break;
    }
    case OR_V_BIPOLAR: { /* 1914-1935: p = -pi/2 * shift */
        double x2y2 = R2SQ, tt = x2y2 + 1.0, x2 = 2.0 * x;
        double yy = 0.5 * atan2(2.0 * y, x2y2 - 1.0) + P[0];
        yy -= M_PI * floor(yy * M_1_PI + 0.5);
        X = log((tt + x2) / (tt - x2)); Y = yy; break;
    }
    case OR_V_BOARDERS: { /* 1940-1983: p = prob */
        double rx = rint(x), ry = rint(y), ox = x - rx, oy = y - ry;
        if (rand_num(rng) >= P[0]) {
            X = ox * 0.5 + rx; Y = oy * 0.5 + ry;
        } else {
            double mag = 1.0 - P[0];
            if (fabs(ox) >= fabs(oy)) {
                double sg = copysign(mag, ox);
                X = ox * 0.5 + rx + sg; Y = oy * 0.5 + ry + sg * oy / ox;
            } else {
                double sg = copysign(mag, oy);
                X = ox * 0.5 + rx + sg * ox / oy; Y = oy * 0.5 + ry + sg;
            }
        }
        break;
    }
    case OR_V_BUTTERFLY: { /* 1988-2003 */
        double y2 = 2.0 * y;
        r = sqrt(fabs(x * y) / (x * x + y2 * y2 + EPS));
        X = x * r; Y = y2 * r; break;
    }
    case OR_V_CELL: { /* 2008-2033: p = size, 1/size */
        double fx = floor(x * P[1]), fy = floor(y * P[1]);
        double dx = x - fx * P[0], dy = y - fy * P[0];
        double xs = copysign(2.0, fx), ys = copysign(2.0, fy);
        double x2 = fx * xs, y2 = fy * ys;
        x2 -= (double)(fx < 0);
        y2 -= (double)(fy < 0);
        X = dx + x2 * P[0]; Y = -dy - y2 * P[0]; break;
    }
    case OR_V_CPOW: { /* 2038-2061: p = va, vc, vd, power */
        a = atan2(y, x);
        double lnr = 0.5 * log(R2SQ);
        double ang = P[1] * a + P[2] * lnr + P[0] * floor(P[3] * rand_num(rng));
        sincos(ang, &s, &c);
        d = exp(P[1] * lnr - P[2] * a);
        X = c * d; Y = s * d; break;
    }
    case OR_V_CURVE: /* 2066-2091: p = xamp, yamp, 1/xlen^2, 1/ylen^2 */
        X = x + P[0] * exp(-y * y * P[2]);
        Y = y + P[1] * exp(-x * x * P[3]); break;
    case OR_V_EDISC: { /* 2096-2120 */
        double tmp = R2SQ + 1.0, tmp2 = 2.0 * x;
        double xmax = 0.5 * (sqrt(tmp + tmp2) + sqrt(tmp - tmp2));
        double a1 = log(xmax + sqrt(xmax - 1.0));
        double a2 = -acos(x / xmax);
        double s1, c1;
        sincos(a1, &s1, &c1);
        double s2 = sinh(a2), c2 = cosh(a2);
        s1 *= copysign(1.0, -y);
        X = c2 * c1; Y = s2 * s1; break;
    }
    case OR_V_ELLIPTIC: { /* 2125-2144 */
        double tmp = R2SQ + 1.0, x2 = 2.0 * x;
        double xmax = 0.5 * (sqrt(tmp + x2) + sqrt(tmp - x2));
        double aa = x / xmax, bb = 1.0 - aa * aa, ssx = xmax - 1.0;
        bb = bb < 0.0 ? 0.0 : sqrt(bb);
        ssx = ssx < 0.0 ? 0.0 : sqrt(ssx);
        X = atan2(aa, bb); Y = copysign(1.0, y) * log(xmax + ssx); break;
    }
    case OR_V_ESCHER: { /* 2149-2171: p = vc, vd */
        a = atan2(y, x);
        double lnr = 0.5 * log(R2SQ);
        double n = P[0] * a + P[1] * lnr;
        sincos(n, &s, &c);
        d = exp(P[0] * lnr - P[1] * a);
        X = c * d; Y = s * d; break;
    }
    case OR_V_FOCI: { /* 2176-2192 */
        double expx = 0.5 * exp(x), expnx = 0.25 / expx;
        sincos(y, &s, &c);
        d = 1.0 / (expx + expnx - c);
        X = (expx - expnx) * d; Y = s * d; break;
    }
    case OR_V_LAZYSUSAN: { /* 2197-2230: p = x, y, spin, twist, space, weight */
        double xx = x - P[0], yy = y + P[1];
        r = hypot(xx, yy);
        if (r < P[5]) {
            a = atan2(yy, xx) + P[2] + P[3] * (P[5] - r);
            sincos(a, &s, &c);
            X = r * c + P[0]; Y = r * s - P[1];
        } else {
            r = 1.0 + P[4] / (r + EPS);
            X = r * xx + P[0]; Y = r * yy - P[1];
        }
        break;
    }
    case OR_V_LOONIE: { /* 2235-2254: p = weight, weight^2 */
        double r2 = R2SQ;
        r = P[0];
        if (r2 < P[1])
            r *= sqrt(P[1] / (r2 + EPS) - 1.0);
        X = x * r; Y = y * r; break;
    }
    case OR_V_OSCOPE: { /* 2259-2281: p = 2 pi freq, amp, damp, sep */
        double damp = exp(-fabs(x) * P[2]);
        double tt = P[1] * damp * cos(P[0] * x) + P[3];
        X = x; Y = copysign(1.0, fabs(y) - tt) * y; break;
    }
    case OR_V_POPCORN: /* 2286-2305: p = x, y, c */
        X = x + P[0] * sin(tan(y * P[2]));
        Y = y + P[1] * sin(tan(x * P[2])); break;
    default:
        X = Y = NAN; break;
    }
#undef R2SQ
#undef R2
#undef ANG
    if (dims == 2) {
        out[0] = X;
        out[1] = Y;
    } else {
        for (i = 0; i < dims; ++i)
            out[i] = 0.0;
        out[v->axis_x] = X;
        out[v->axis_y] = Y;
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

/*
 * ORACLE -- test infrastructure only (see chaos_oracle.c).  Flat flame
 * description filled by oracle/flame_oracle.py through ctypes.
 */
#ifndef CHAOS_ORACLE_H
#define CHAOS_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#define OR_MAXD 4          /* dimensions 1..4 (ffr-buf compiles 1..3; BufferRenderer<4> for 4) */
#define OR_MAXC 128        /* color_dimensions <= 127 (flame.hpp:156) */
#define OR_MAXX 4096       /* xform ids reported in or_stats */
#define OR_NPARAM 16

/* variation ids: index in the oracle's name table (flame_oracle.py) */
enum {
    OR_V_LINEAR = 0,
    OR_V_SINUSOIDAL = 1,
    OR_V_SPHERICAL = 2,
    OR_V_BENT = 3,
    OR_V_RECTANGLES = 4,
    OR_V_FISHEYE = 5,
    OR_V_BUBBLE = 6,
    OR_V_NOISE = 7,
    OR_V_BLUR = 8,
    OR_V_GAUSSIAN_BLUR = 9,
    OR_V_SQUARE_NOISE = 10,
    OR_V_SEPARATION = 11,
    OR_V_SPLITS = 12,
    OR_V_PRE_BLUR = 13,
    OR_V_MODULUS = 14,
    OR_V_CELLN = 15,
    OR_V_SPHERICAL_P = 16,
    OR_V_UNIT_SPHERE = 17,
    OR_V_UNIT_SPHERE_P = 18,
    OR_V_UNIT_CUBE = 19,
    OR_V_SWIRL = 20,
    OR_V_HORSESHOE = 21,
    OR_V_POLAR = 22,
    OR_V_POLAR2 = 23,
    OR_V_HANDKERCHIEF = 24,
    OR_V_HEART = 25,
    OR_V_DISC = 26,
    OR_V_DISC2 = 27,
    OR_V_WAVES = 28,
    OR_V_FAN = 29,
    OR_V_RINGS = 30,
    OR_V_SPIRAL = 31,
    OR_V_HYPERBOLIC = 32,
    OR_V_DIAMOND = 33,
    OR_V_EX = 34,
    OR_V_JULIA = 35,
    OR_V_EXPONENTIAL = 36,
    OR_V_POWER = 37,
    OR_V_COSINE = 38,
    OR_V_BLOB = 39,
    OR_V_PDJ = 40,
    OR_V_CYLINDER = 41,
    OR_V_PERSPECTIVE = 42,
    OR_V_JULIAN = 43,
    OR_V_JULIASCOPE = 44,
    OR_V_RADIAL_BLUR = 45,
    OR_V_PIE = 46,
    OR_V_NGON = 47,
    OR_V_CURL = 48,
    OR_V_ARCH = 49,
    OR_V_TANGENT = 50,
    OR_V_RAYS = 51,
    OR_V_BLADE = 52,
    OR_V_SECANT = 53,
    OR_V_TWINTRIAN = 54,
    OR_V_CROSS = 55,
    OR_V_EXP = 56,
    OR_V_LOG = 57,
    OR_V_SIN = 58,
    OR_V_COS = 59,
    OR_V_TAN = 60,
    OR_V_SEC = 61,
    OR_V_CSC = 62,
    OR_V_COT = 63,
    OR_V_SINH = 64,
    OR_V_COSH = 65,
    OR_V_TANH = 66,
    OR_V_SECH = 67,
    OR_V_CSCH = 68,
    OR_V_COTH = 69,
    OR_V_AUGER = 70,
    OR_V_FLUX = 71,
    OR_V_MOBIUS = 72,
    OR_V_SCRY = 73,
    OR_V_SPLIT = 74,
    OR_V_STRIPES = 75,
    OR_V_WEDGE = 76,
    OR_V_WEDGE_JULIA = 77,
    OR_V_WEDGE_SPH = 78,
    OR_V_WHORL = 79,
    OR_V_SUPERSHAPE = 80,
    OR_V_FLOWER = 81,
    OR_V_CONIC = 82,
    OR_V_PARABOLA = 83,
    OR_V_BIPOLAR = 84,
    OR_V_BOARDERS = 85,
    OR_V_BUTTERFLY = 86,
    OR_V_CELL = 87,
    OR_V_CPOW = 88,
    OR_V_CURVE = 89,
    OR_V_EDISC = 90,
    OR_V_ELLIPTIC = 91,
    OR_V_ESCHER = 92,
    OR_V_FOCI = 93,
    OR_V_LAZYSUSAN = 94,
    OR_V_LOONIE = 95,
    OR_V_OSCOPE = 96,
    OR_V_POPCORN = 97,
    OR_V_COUNT = 98,
    OR_FIRST_2D = 20
};

typedef struct {
    int32_t type;
    int32_t axis_x, axis_y, rng_draws;
    double weight;
    double params[OR_NPARAM];
} or_var;

typedef struct {
    uint64_t id;
    double weight;
    int32_t has_pre, has_post;
    double pre_A[OR_MAXD * OR_MAXD], pre_b[OR_MAXD];
    double post_A[OR_MAXD * OR_MAXD], post_b[OR_MAXD];
    int32_t var_begin, var_count;
    int32_t has_color, pad;
    double color_speed;
} or_xform;

typedef struct {
    int32_t dims, nxf, has_final, color_dims;
    int32_t xform_ids, pad;
    uint64_t size[OR_MAXD];
    double lo[OR_MAXD], hi[OR_MAXD];
    const or_xform *xf;       /* nxf sorted xforms, then the final xform */
    const or_var *vars;
    const double *colors;     /* (nxf + 1) * color_dims */
    const double *xfcw;       /* nxf cumulative weights */
} or_flame;

typedef struct {
    int32_t ok, pad;
    uint64_t s_iter, s_plot, bad, dropped;
    double ext_lo[OR_MAXD], ext_hi[OR_MAXD];
    uint64_t xf_dist[OR_MAXX];
} or_stats;

size_t oracle_isaac_state_bytes(void);
void oracle_isaac_seed(void *state, uint64_t key);
void oracle_isaac_words(uint64_t key, uint64_t n, uint64_t *out);
uint64_t oracle_fmix64(uint64_t k);
uint64_t oracle_stream_key(uint64_t seed, uint64_t stream);
void oracle_index_mults(const or_flame *f, double *mult_d, uint64_t *mult_i,
    uint64_t *cells);
int oracle_pick_sequence(const or_flame *f, uint64_t key, uint64_t n,
    int32_t *out);
int oracle_step(const or_flame *f, int xf_index, uint64_t key, uint64_t npts,
    const double *in, double *out);
int oracle_render(const or_flame *f, uint64_t seed, uint64_t streams,
    uint64_t samples, uint64_t traj_len, uint64_t settle, uint64_t bad_limit,
    int threads, uint64_t *counts, double *colors, or_stats *out);
int oracle_variation_words(int type, int dims);
int oracle_trace(const or_flame *f, uint64_t key, uint64_t settle, uint64_t n,
    int32_t *ids, double *pts);

#endif

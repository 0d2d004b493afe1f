/*
 * ORACLE -- test infrastructure only (see chaos_oracle.c).  Flat flame
 * description filled by oracle/flame_oracle.py through ctypes.
 */
#ifndef CHAOS_ORACLE_H
#define CHAOS_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#define OR_MAXD 3          /* dimensions compiled into ffr-buf: 1, 2, 3 */
#define OR_MAXC 128        /* color_dimensions <= 127 (flame.hpp:156) */
#define OR_MAXX 4096       /* xform ids reported in or_stats */
#define OR_NPARAM 16

/* variation ids: index in the oracle's name table (flame_oracle.py) */
enum {
    OR_V_LINEAR = 0,
    OR_V_SINUSOIDAL = 1,
    OR_V_SPHERICAL = 2,
    OR_V_SWIRL = 20,
    OR_V_HORSESHOE = 21,
    OR_V_POLAR = 22,
    OR_V_JULIA = 35
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
int oracle_trace(const or_flame *f, uint64_t key, uint64_t settle, uint64_t n,
    int32_t *ids, double *pts);

#endif

/*
 * ffr_wire.h -- request/response framing of ffr-serve, the network front
 * end of the serving loop (ffr_server_* in ffr_gpu.h).  No reference
 * counterpart: the reference has no serving mode; its interchange formats
 * are the flame JSON (FLAME_JSON.md) and the raw buffer file
 * (src/renderers/buffer_renderer.hpp:476-480), and both travel unchanged
 * inside these frames.
 *
 * A connection carries requests and responses strictly in turn.  All
 * integers are little-endian; the structs below are packed by construction
 * (naturally aligned fields, no padding).
 *
 * Request:  ffr_wire_request, then json_len bytes of flame JSON, then
 *           init_len bytes of an initial buffer (file layout).
 * Response: ffr_wire_response, then payload_len bytes: the job's buffer in
 *           the file layout (FFR_WIRE_READ, or FFR_WIRE_WAIT with
 *           FFR_WIRE_WITH_BUFFER), or the error message when status is not
 *           FFR_OK / FFR_BAD_VALUES.
 */
#ifndef FFR_WIRE_H
#define FFR_WIRE_H

#include <stdint.h>

#define FFR_WIRE_VERSION 1

enum ffr_wire_op {
    FFR_WIRE_SUBMIT = 1,    /* json (+ init), samples, seed, bad_limit -> job */
    FFR_WIRE_CONTINUE = 2,  /* job = parent, samples, seed, bad_limit -> job */
    FFR_WIRE_WAIT = 3,      /* job, timeout_ms; flags: FFR_WIRE_WITH_BUFFER */
    FFR_WIRE_READ = 4,      /* job -> buffer */
    FFR_WIRE_POLL = 5,      /* job -> state */
    FFR_WIRE_CANCEL = 6,    /* job */
    FFR_WIRE_RELEASE = 7,   /* job */
    FFR_WIRE_SHUTDOWN = 8   /* stop the serving loop and exit */
};

enum { FFR_WIRE_WITH_BUFFER = 1 };

typedef struct ffr_wire_request {
    char magic[4];          /* "FFRQ" */
    uint32_t version;       /* FFR_WIRE_VERSION */
    uint32_t op;            /* ffr_wire_op */
    uint32_t flags;
    uint64_t job;           /* parent (CONTINUE) or job */
    uint64_t samples;
    uint64_t seed;
    uint64_t bad_limit;
    uint64_t timeout_ms;    /* WAIT: 0 = no limit */
    uint64_t json_len;
    uint64_t init_len;
} ffr_wire_request;         /* 72 bytes */

typedef struct ffr_wire_response {
    char magic[4];          /* "FFRR" */
    uint32_t status;        /* ffr_status of the request */
    uint64_t job;
    uint32_t state;         /* FFR_JOB_* (ffr_job_info) */
    uint32_t job_status;    /* the job's own ffr_status once finished */
    uint64_t samples;
    uint64_t buffer_bytes;
    uint64_t parent;
    uint64_t submit_ns;
    uint64_t admit_ns;
    uint64_t done_ns;
    uint64_t payload_len;
} ffr_wire_response;        /* 80 bytes */

#endif /* FFR_WIRE_H */

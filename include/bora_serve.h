/* Serving layer over the FLIP substep: many independent simulations of uneven sizes on
 * one GPU, admitted continuously against a device-memory budget.
 *
 * The reference has no counterpart: its only caller, the Houdini node SOP_FlipWater
 * (houdini/source/SOP_FlipWater.cpp:80-363), drives one FLIPMethod per cook. This API
 * serves a stream of requests, each "advance this particle set by N substeps":
 *
 *   - bora_serve_submit queues a request (the particles are copied; the call returns at
 *     once) and returns its id;
 *   - a scheduler thread admits queued requests in arrival order whenever a slot is free
 *     and the request's device-memory estimate fits in the budget next to the requests
 *     already running (a request that alone exceeds the budget fails);
 *   - a stepper thread advances all running requests together, one round at a time:
 *     every running request takes one step per round, through bora_flip_step_batch, so the
 *     pressure solve's kernels (almost all of a step's launches) run once per round for
 *     all requests, each request on its own tiles and reductions; a request that arrives
 *     while others run joins at the next round as soon as a slot and memory free up
 *     (continuous batching, not a queue drained in rounds);
 *   - finished requests keep their final particles (and per-step latencies) until
 *     bora_serve_release.
 *
 * A request's launches and arithmetic in a batched step do not depend on the other
 * requests, so its result is bit-identical whether it runs alone or in a mix.
 *
 * All functions return a bora_flip.h status code (BORA_OK = 0, negative = error).
 */
#ifndef BORA_SERVE_H
#define BORA_SERVE_H

#include <stddef.h>
#include <stdint.h>

#include "bora_flip.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct bora_server* bora_serve_handle;

typedef struct bora_serve_config
{
    uint64_t hbm_budget_bytes; /* device memory the running requests may hold together */
    int max_running;           /* running requests at most (default 64) */
    int reserved;
} bora_serve_config;

/* bora_serve_wait: the request did not finish within the timeout */
#define BORA_WARN_TIMEOUT 2

/* request states */
#define BORA_REQ_QUEUED 0
#define BORA_REQ_RUNNING 1
#define BORA_REQ_DONE 2
#define BORA_REQ_FAILED 3

typedef struct bora_serve_request_status
{
    int state;                 /* BORA_REQ_* */
    int status;                /* bora_flip status of a failed request, else BORA_OK */
    int steps_total;
    int steps_done;
    uint64_t num_particles;    /* live particles (after the last step taken) */
    uint64_t estimate_bytes;   /* device-memory estimate used for admission */
    uint64_t device_bytes;     /* device memory the request held (peak) */
    double queued_s;           /* submit -> admit (s) */
    double run_s;              /* admit -> done (s) */
    double step_ms_p50;        /* per-step wall latency of this request */
    double step_ms_p99;
    double step_ms_max;
} bora_serve_request_status;

typedef struct bora_serve_stats
{
    uint64_t submitted, admitted, done, failed;
    int queued, running;
    uint64_t bytes_reserved;   /* estimates of the running requests */
    uint64_t bytes_reserved_peak;
    int running_peak;
    int reserved;
    uint64_t particle_steps;   /* over finished requests */
    uint64_t steps;            /* substeps over finished requests */
    double step_ms_p50;        /* per-step wall latency over all finished requests */
    double step_ms_p99;
    double step_ms_max;
} bora_serve_stats;

/* Default configuration: 120 GB budget, 16 running requests. */
int bora_serve_default_config( bora_serve_config* out );

/* Start a server on the current device (its scheduler thread starts at once). */
int bora_serve_create( const bora_serve_config* cfg, bora_serve_handle* out );

/* Wait for every admitted request to finish, drop queued ones, release everything. */
int bora_serve_destroy( bora_serve_handle h );

/* Queue a request: advance n particles (pos, vel: n x 3 floats, `space` as in
 * bora_flip_set_particles) by `steps` substeps of `dt` on the given grid. The grid and
 * parameters are copied, as are the particles. */
int bora_serve_submit( bora_serve_handle h, const bora_grid_desc* grid, const bora_flip_params* params,
                       const float* pos, const float* vel, size_t n, int space, int steps, float dt,
                       uint64_t* request_id );

/* Optional static colliders for a queued request (same layout as bora_flip_set_colliders). */
int bora_serve_set_colliders( bora_serve_handle h, uint64_t request_id, const float* boxes, int count, float band );

int bora_serve_poll( bora_serve_handle h, uint64_t request_id, bora_serve_request_status* out );

/* Block until the request is done or failed (timeout_s < 0: no limit). Returns
 * BORA_ERR_INVALID_ARG for an unknown id and BORA_WARN_TIMEOUT on timeout. */
int bora_serve_wait( bora_serve_handle h, uint64_t request_id, double timeout_s );

/* Final particles of a finished request, in the space it was submitted in (ids in
 * ascending order). *n receives the count; capacity is in particles. */
int bora_serve_result( bora_serve_handle h, uint64_t request_id, float* pos, float* vel, int32_t* ids,
                       size_t capacity, size_t* n );

/* Forget a finished request (its results and latencies). */
int bora_serve_release( bora_serve_handle h, uint64_t request_id );

/* Block until nothing is queued or running. */
int bora_serve_drain( bora_serve_handle h );

int bora_serve_get_stats( bora_serve_handle h, bora_serve_stats* out );

/* Device-memory estimate the scheduler uses for a request (bytes). */
uint64_t bora_serve_estimate_bytes( const bora_grid_desc* grid, size_t n, int solver );

#ifdef __cplusplus
}
#endif

#endif /* BORA_SERVE_H */

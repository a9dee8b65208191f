/*
 * mara_batch.h -- C ABI of the batched, continuously refilled form of the
 * time step: many independent Newtonian-hydro grids of uneven sizes (1-D and
 * 2-D) resident on one GPU, advanced together over a tile list that spans
 * all of them, each grid with its own dt = min(cfl * Courant, t_final - t)
 * (the reference's driver loop, src/Problems.cpp:181-188, per grid).  With
 * `persistent` set, a batch step (every RK stage over both tile lists) is
 * one cooperative launch with grid-wide barriers between the stages;
 * otherwise each stage is a launch per tile list and the step is captured
 * once as a CUDA graph.  Both forms give the same bits.  Admitting and
 * retiring grids edits device-resident tables only.
 *
 * There is no counterpart of the batch in the reference (its drivers run
 * one MeshData at a time); each grid's arithmetic is the mixed-precision
 * MethodOfLinesTVD::advance of mara_gpu.h, and does not depend on which
 * other grids share the batch or on where its tiles land.
 */
#ifndef MARA_BATCH_H
#define MARA_BATCH_H

#include <stdint.h>

#include "mara_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

enum {
    MARA_ERR_NO_ROOM = 36   /* the HBM budget or the grid table is full */
};

enum {
    MARA_TILE_AUTO = 0      /* the default tile shape (1-D: 256 zones, 2-D:
                               32x16); the autotuner (mara2_gb300.batch.
                               autotune) measures the others on the request
                               mix and its caller passes the fastest */
};

typedef struct MaraBatchConfig {
    int device;
    int64_t hbm_budget_bytes;  /* bytes of grid state the batch may hold     */
    int max_grids;             /* slots in the grid table                   */
    int max_zones_per_grid;    /* staging size for uploads / downloads      */
    int recon;                 /* MARA_RECON_PCM or MARA_RECON_PLM          */
    int riemann;               /* MARA_RIEMANN_*                            */
    int rk_order;              /* 1, 2, 3                                   */
    int tile_1d;               /* zones per 1-D tile: 128, 256, 512, 0=256  */
    int tile_2d;               /* 2-D tile: 0=32x16, 1=32x8, 2=32x16, 3=64x8,
                                  4=32x16 one face per thread (PLM faces
                                  otherwise go in runs along their normal) */
    int lockstep_1d;           /* 1: small 1-D grids step with the tile lists
                                  (0: on thread-block clusters, see below)  */
    int persistent;            /* 1: one cooperative launch per batch step
                                  (1-D tiles of 256 or 512 zones, 2-D tiles
                                  32x8 or 32x16; other shapes keep the
                                  per-stage launches)                       */
    int ctas_per_sm;           /* CTAs per SM of that launch; 0 = as many as
                                  the kernel's resources allow              */
} MaraBatchConfig;

typedef struct MaraBatchStats {
    int active;                /* grids resident and not yet finished       */
    int finished;              /* grids finished and not yet retired        */
    int64_t zones;             /* interior zones of the active grids        */
    int64_t bytes_in_use;      /* grid state held against the budget        */
    int64_t zone_updates;      /* zone-updates done since creation          */
    int64_t steps;             /* batch steps enqueued                      */
    int64_t kernel_launches;
} MaraBatchStats;

typedef struct MaraBatch MaraBatch;

int mara_batch_create(const MaraBatchConfig* config, MaraBatch** batch);
int mara_batch_destroy(MaraBatch* batch);

/* Admit one grid (law must be MARA_LAW_HYDRO, 1-D or 2-D; recon / riemann /
 * rk_order must match the batch).  P_aos is the host MeshData::P (FP64 AoS
 * with guards).  Returns MARA_ERR_NO_ROOM when the grid's state does not fit
 * the remaining budget or no slot is free; *slot receives the grid's slot. */
int mara_batch_admit(MaraBatch* b, const MaraGpuConfig* grid, const double* P_aos, double t_final, double cfl,
                     int* slot);

/* Enqueue `steps` batch steps: every active grid advances one time step with
 * its own dt; grids that reach t_final stop.  Asynchronous.
 *
 * Unless lockstep_1d is set, a 1-D grid of at most 8192 zones is not in the
 * tile lists: it runs its own driver loop on a thread-block cluster that
 * holds it in shared memory, on a side stream concurrent with the batch
 * steps.  Each call advances such a grid by a number of steps adapted so
 * that the clusters take about as long as the call's batch steps (by 1024
 * when no grid is in the tile lists).  Its results are the same bits. */
int mara_batch_step(MaraBatch* b, int steps);

/* Wait for the enqueued steps and list the slots that have reached t_final
 * since the last poll (up to cap). */
int mara_batch_poll(MaraBatch* b, int* slots, int cap, int* n);

/* Copy a finished grid's primitives (FP64 AoS with guards) to the host, its
 * time and step count, and free its slot and memory. */
int mara_batch_retire(MaraBatch* b, int slot, double* P_aos, double* t, int64_t* steps);

int mara_batch_stats(MaraBatch* b, MaraBatchStats* stats);

/* The tile shapes in use (as configured, or the defaults). */
int mara_batch_tiles(MaraBatch* b, int* tile_1d, int* tile_2d);

/* The launch form in use: *persistent = 1 with *ctas CTAs in the one
 * cooperative launch per step, or 0 with *ctas CTAs per 2-D stage launch.
 * No counterpart in the reference (it has no batch). */
int mara_batch_launch_form(MaraBatch* b, int* persistent, int* ctas);

#ifdef __cplusplus
}
#endif
#endif

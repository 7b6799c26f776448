/*
 * ofd.h — C ABI of the GB300 device runtime for the opesci-fd elastic
 * velocity-stress hot path (libofd.so).
 *
 * The reference has no device runtime: its generated program
 * (opesci/templates/regular3d_tmpl.py:41-118, emitted sample
 * benchmarks/test3d.cpp) allocates the nine fields, runs the OpenMP time loop
 * inside extern "C" opesci_execute() and computes error norms inside
 * opesci_convergence().  This header is the device-side replacement of that
 * generated body: the CUDA program emitted by opesci/templates/cuda_tmpl.py
 * keeps the reference's three entry points and implements them on top of the
 * calls below, and the batching/serving drivers call them directly.
 *
 * Conventions
 *  - every call returns 0 on success or a negative OFD_E* code; the message of
 *    the last failure on the calling thread is returned by ofd_last_error();
 *  - host arrays use the reference layout float[dim1][dim2][dim3] (z fastest,
 *    margins included), the layout of one time level of the reference's
 *    real_t[2][dim1][dim2][dim3] field arrays (regulargrid.py:466-496);
 *  - field numbers follow the reference's OpesciGrid order, velocities then
 *    stresses (staggeredgrid.py:69-71): U V W Txx Tyy Tzz Txy Tyz Txz;
 *  - one CUDA stream per handle; calls on one handle are not re-entrant,
 *    different handles are independent;
 *  - transient device scratch (media preprocessing, transfers of 16-bit and
 *    FP64 fields) comes from a stream-ordered pool of the library, one per
 *    device, which keeps up to 4 GiB mapped between calls; ofd_footprint
 *    does not count it.
 */
#ifndef OFD_H
#define OFD_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OFD_OK 0
#define OFD_EINVAL (-1)    /* bad argument or unsupported configuration */
#define OFD_ECUDA (-2)     /* a CUDA call failed */
#define OFD_ENOMEM (-3)    /* device allocation failed */
#define OFD_ESTATE (-4)    /* call not valid in the handle's current state */
#define OFD_ETIMEOUT (-5)  /* a bounded device wait expired */

enum ofd_field { OFD_U = 0, OFD_V, OFD_W, OFD_TXX, OFD_TYY, OFD_TZZ, OFD_TXY, OFD_TYZ, OFD_TXZ, OFD_NFIELDS };

enum ofd_storage { OFD_F32 = 0, OFD_F16 = 1, OFD_BF16 = 2, OFD_F64 = 3 };

/* free-surface algorithm per face (staggeredgrid.py:214-232) */
enum ofd_face_bc { OFD_BC_NONE = 0, OFD_BC_LEVANDER = 1, OFD_BC_ROBERTSSON = 2 };

typedef struct ofd_config {
    int dim[3];            /* dim1, dim2, dim3 = interior points + 2*margin */
    int space_order;       /* 2, 4, 6 or 8; margin = space_order/2 */
    int storage;           /* enum ofd_storage; arithmetic is FP32 (FP64 for OFD_F64) */
    int legacy_bc;         /* 1: omit the Levander normal-stress recompute (older generator) */
    int free_surface[6];   /* enum ofd_face_bc for faces x-, x+, y-, y+, z-, z+ */
    double spacing[3];     /* dx1, dx2, dx3 */
    double dt;
    double weights[4];     /* staggered first-derivative weights c_1..c_R (R = space_order/2) */
    float field_scale[9];  /* stored = value * scale (16-bit storage; powers of two; 0 = 1) */
    int kernel_variant;    /* 0 = best available, 1 = plain (one thread per column) */
    int rounding;          /* 16-bit storage: enum ofd_rounding of the sweeps' stores */
} ofd_config;

/* Rounding of the values the sweeps store in 16-bit fields (no counterpart in
 * the reference, which stores float or double).  Stochastic rounding stores
 * the upper neighbour of v with probability (v - lower) / (upper - lower),
 * from a deterministic hash of (element, field, step): the same bits on every
 * kernel path and run, and v in expectation, so increments below half a unit
 * in the last place are not lost.  Ghost cells and the source use
 * round-to-nearest.  FP32 and FP64 storage ignore the mode. */
enum ofd_rounding { OFD_ROUND_NEAREST = 0, OFD_ROUND_STOCHASTIC = 1 };

typedef struct ofd_handle ofd_handle;

/* Device for handles created afterwards by the calling thread (no
 * counterpart in the reference, which runs on the host).  The library
 * carries its own CUDA runtime, so a device chosen through another runtime
 * (a framework's) does not apply to it; one process per GPU calls this with
 * its local rank. */
int ofd_set_device(int device);

/* Lifecycle.  ofd_create allocates two time levels of the nine fields and the
 * eight effective-media arrays on the current device, all zero. */
int ofd_create(const ofd_config *cfg, ofd_handle **out);
int ofd_destroy(ofd_handle *h);
const char *ofd_last_error(void);
/* bytes ofd_create would allocate for cfg (fields + media), for admission control */
int ofd_footprint(const ofd_config *cfg, size_t *bytes);

/* Media.  Constant media as the reference prints them (beta, lambda, mu;
 * staggeredgrid.py:278-282), or raw rho/vp/vs arrays in the reference layout
 * (the arrays opesci_read_simple_binary_ptr fills, src/opesciIO.cpp:319-342)
 * from which beta, lambda, mu and the averaged beta1..3, mu12, mu13, mu23 of
 * staggeredgrid.py:571-597 are computed on the device. */
int ofd_set_media_const(ofd_handle *h, float beta, float lambda, float mu);
int ofd_set_media(ofd_handle *h, const float *rho, const float *vp, const float *vs);
/* ofd_set_media queued on the handle's stream without waiting (no
 * counterpart in the reference): the arrays (host or device memory) must stay
 * valid until the stream reaches the copy; pinned host memory makes the copy
 * asynchronous.  ofd_sync waits for it. */
int ofd_set_media_async(ofd_handle *h, const float *rho, const float *vp, const float *vs);

/* Literal tables of the generated update expressions (required before
 * ofd_step).  The sweeps evaluate the reference generator's expanded,
 * constant-folded stencil expression (staggeredgrid.py:728-748 through
 * regulargrid.py:329-342 and codeprinter.py) term by term in its printed
 * order; ks/kv hold the values of its floating literals in order of
 * appearance, as opesci.templates.cuda_gen.sweep_tables computes them.
 * het = 1 for media read from arrays (media are factors of each term), 0 for
 * constant media folded into the literals.  nks/nkv must equal the table
 * sizes of the prebuilt expression for this space order and media mode. */
int ofd_set_coefficients(ofd_handle *h, int het, const float *ks, int nks, const float *kv, int nkv);
/* Literal table of the generated space-order-4 Levander ghost expressions
 * (the frontend's ghost equations fields.py:192-381 as staggeredgrid.py:754-864
 * applies them, printed like the update expressions; values as
 * opesci.templates.cuda_gen.ghost_table computes them).  With it the ghost
 * cells are evaluated from those printed expressions, term for term; without
 * it (or nkg = 0) from restated formulas that agree to rounding.  Needs
 * space order 4, Levander free surfaces on all six faces, FP32/FP16/BF16
 * storage and ofd_set_coefficients of the same media mode first. */
int ofd_set_ghost_coefficients(ofd_handle *h, int het, const float *kg, int nkg);

/* Field transfer, reference layout, host memory (pageable or pinned); the
 * calls return once the copy is complete.  The reference publishes its host
 * arrays through OpesciGrid after opesci_execute (regulargrid.py:445-464),
 * which the generated program's opesci_execute does with these calls. */
int ofd_upload_field(ofd_handle *h, int field, int level, const float *host);
int ofd_download_field(ofd_handle *h, int field, int level, float *host);
/* The same for OFD_F64 storage with double host arrays, exact both ways: the
 * reference's double switch (regulargrid.py:27-28) publishes double arrays.
 * Other storage types report OFD_EINVAL. */
int ofd_upload_field_f64(ofd_handle *h, int field, int level, const double *host);
int ofd_download_field_f64(ofd_handle *h, int field, int level, double *host);
/* The same queued on the handle's stream without waiting (no counterpart in
 * the reference): several fields' copies then run back to back, and with
 * pinned host memory they overlap other host work.  The host array must stay
 * valid (and, for downloads, unread) until ofd_sync returns. */
int ofd_upload_field_async(ofd_handle *h, int field, int level, const float *host);
int ofd_download_field_async(ofd_handle *h, int field, int level, float *host);
/* Same with device memory in the reference layout. */
int ofd_upload_field_device(ofd_handle *h, int field, int level, const float *dev);
int ofd_download_field_device(ofd_handle *h, int field, int level, float *dev);
int ofd_zero_fields(ofd_handle *h);

/* Point source: after every step, Txx[src] -= wx[step]/3, Tyy[src] -=
 * wy[step]/3 and Tzz[src] -= wz[step]/3 while step < nt: the reference driver's
 * x, y and z source signals (tests/src/test_ref_iso_elastic.cpp:100-126,274-290).
 * (sx, sy, sz) is an array index including margins; nt <= 0 or a null signal
 * removes the source.  The signals are copied; the call waits for the copy. */
int ofd_set_source_xyz(ofd_handle *h, int sx, int sy, int sz, const float *wx, const float *wy, const float *wz,
                       int nt);
/* The same with one signal for all three normal stresses. */
int ofd_set_source(ofd_handle *h, int sx, int sy, int sz, const float *wavelet, int nt);

/* Receivers (seismograms; the reference records them in its hand-written
 * driver, tests/src/test_ref_iso_elastic.cpp:227-270, reading positions with
 * opesci_read_receivers, src/opesciIO.cpp:372-396).  ijk: 3*nrec array
 * indices (x, y, z, margins included).  After every step, once its ghosts
 * and source are applied, row (step - 1) of a device buffer
 * traces[nt_cap][4][nrec] receives U, V, W and P = (Txx + Tyy + Tzz) / 3 of
 * the new level; steps beyond nt_cap are not recorded.  nrec = 0 removes the
 * receivers.  The buffer starts at zero. */
int ofd_set_receivers(ofd_handle *h, int nrec, const int *ijk, int nt_cap);
/* copy the whole trace buffer (nt_cap * 4 * nrec floats) to host memory */
int ofd_get_traces(ofd_handle *h, float *host);

/* SEG-Y earth model decoding (the reference's opesci_read_model_segy,
 * src/opesciIO.cpp:419-612, format code 1): file is the whole SEG-Y image in
 * host memory, (nx, ny, nz) traces per record, records and samples per trace
 * from its header, swap_endian whether the header was read byte-swapped.
 * The IBM-float samples are decoded on the device into out[nz][ny][nx] (host
 * memory, x fastest, the reference's array order).  No handle needed. */
int ofd_segy_decode_ibm(const void *file, long file_size, int nx, int ny, int nz, int swap_endian, float *out);

/* Write name.vts: a VTK XML structured grid of one host field of
 * dims[0] x dims[1] x dims[2] floats (last index fastest), as the reference's
 * opesci_dump_field_vts_3d (src/opesciIO.cpp:614-667) does for the generated
 * code's output_vts step (opesci/regulargrid.py:702-719): point coordinates
 * (index - margin) * spacing in the reference's insertion order, one
 * point-data array "field".  Appended raw data, UInt64 headers, no
 * compression.  Host only; no handle or GPU needed. */
int ofd_write_field_vts_3d(const char *name, const int dims[3], const float spacing[3], int margin,
                           const float *field);

/* Ghost cells of one level as the reference's initialise_bc does for the
 * initial level (staggeredgrid.py:866-879): stress mirrors, then velocity
 * ghosts. */
int ofd_apply_boundary_init(ofd_handle *h, int level);

/* Advance nsteps time steps (staggered3d_tmpl.py:40-58 loop body): stress
 * sweep, stress ghosts, velocity sweep, velocity ghosts, source.  Asynchronous
 * on the handle's stream. */
int ofd_step(ofd_handle *h, int nsteps);
int ofd_sync(ofd_handle *h);
/* Non-blocking: 0 when all work queued on the handle has finished, 1 while
 * some is still running, < 0 on error (serving loops poll with it). */
int ofd_query(ofd_handle *h);
/* ofd_step with CUDA events recorded on the handle's stream around every
 * kernel class of every step; waits for completion.  ms_total is the time
 * from the first to the last event; ms_class[k] the summed device time of
 * class k: 0 stress sweep, 1 stress ghosts, 2 velocity sweep, 3 velocity
 * ghosts and source.  launches (may be NULL) receives the kernel count. */
int ofd_step_profiled(ofd_handle *h, int nsteps, double *ms_total, double ms_class[4], long *launches);
/* ofd_step through a cached CUDA graph of two steps (one per starting
 * parity), replayed nsteps/2 times; an odd remainder runs as a plain step.
 * The source index is read on the device, so replays stay exact.  The graph
 * is rebuilt after ofd_set_coefficients, ofd_set_source or ofd_set_tuning. */
int ofd_step_graph(ofd_handle *h, int nsteps);
/* Launch knobs chosen by the autotuner (opesci.autotune), no counterpart in
 * the reference (which tuned Pluto tile sizes, tests/pluto_tile_test.py):
 * per-sweep kernel (0 TMA-tiled, 1 plain), x-chunking multiplier (CTA waves,
 * 1..64), plain-kernel block shape (bx multiple of 32, bx*by <= 256). */
int ofd_set_tuning(ofd_handle *h, int stress_variant, int velocity_variant, int chunk_waves, int plain_bx,
                   int plain_by);
/* Limit of every device-side wait of the handle's kernels (no counterpart in
 * the reference, whose OpenMP loop has no device waits): the TMA pipeline
 * waits of the tiled sweeps and the grid barriers of persistent stepping.
 * A wait that runs out sets the handle's error word, its kernel drains the
 * copies it has in flight and returns, and the next ofd_sync (or timed or
 * profiled step) reports OFD_ETIMEOUT; the context stays usable.  Default
 * 10 s; seconds in (0, 600].  Cached graphs are rebuilt. */
int ofd_set_wait_limit(ofd_handle *h, double seconds);
/* Schedule of the generated space-order-4 ghosts' normal-stress recompute
 * (no counterpart in the reference, which evaluates it inside its ghost
 * loops): mode 0 runs it on the handle's stream after the stress sweep,
 * mode 1 (default) on a second stream at the highest priority beside the
 * stress sweep (ofd_set_ghost_coefficients creates that stream);
 * blocks_per_sm in [1, 16] (default 4) sizes its grid (128-thread blocks).
 * Results are identical in every setting.  Cached graphs are rebuilt. */
int ofd_set_ghost_schedule(ofd_handle *h, int mode, int blocks_per_sm);
/* Persistent time stepping (no counterpart in the reference): when enabled,
 * ofd_step and ofd_step_graph run up to 1024 whole steps per cooperative
 * launch, with grid barriers between the phases of a step.  For small grids,
 * whose steps are shorter than the launches they would otherwise need.
 * Results are identical to the per-kernel path. */
int ofd_set_persistent(ofd_handle *h, int enable);

/* Groups (no counterpart in the reference, which runs one model per
 * process): many independent simulations advanced together, each phase of a
 * step one launch over every member (8 launches per step for the whole
 * group, captured in a two-step CUDA graph).  Members must share the space
 * order, storage and media mode, stand at the same time level, and be large
 * enough for the tiled sweeps (interior >= 32 along z, >= 8 along y); grids,
 * step counts, media, sources and coefficients may differ.  The group copies
 * the members' arguments when it is created: configure members first, and
 * do not destroy a member before its group.  chunk_planes: x planes per
 * sweep CTA (0: the single-handle heuristic).  ofd_group_step orders itself
 * after work already queued on the members' streams and before work queued
 * on them later; it advances every member's step count.  Results equal
 * stepping each member alone. */
typedef struct ofd_group ofd_group;
int ofd_group_create(ofd_handle *const *members, int n, int chunk_planes, ofd_group **out);
/* 1 when the handle may join a group (coefficients set, grid large enough
 * for the tiled sweeps), 0 when not, negative on error */
int ofd_group_eligible(ofd_handle *h);
int ofd_group_step(ofd_group *g, int nsteps);
/* 0 = idle, 1 = busy (non-blocking) */
int ofd_group_query(ofd_group *g);
/* waits, then reports OFD_ETIMEOUT if a member's bounded device wait expired */
int ofd_group_sync(ofd_group *g);
int ofd_group_destroy(ofd_group *g);

/* ofd_step bracketed by CUDA events on the handle's stream (no events
 * between kernels); waits; ms = elapsed time, launches (may be NULL) =
 * kernels run. */
int ofd_step_timed(ofd_handle *h, int nsteps, double *ms, long *launches);

/* completed steps; the newest level is steps % 2 */
int ofd_get_step(ofd_handle *h, long *steps);
int ofd_set_step(ofd_handle *h, long steps);

/* FP64 sum of squares of each field over the interior [m, dim-m)^3 of a level. */
int ofd_field_sumsq(ofd_handle *h, int level, double out[9]);
/* Largest magnitude of each field over the interior of a level (no
 * counterpart in the reference: used to choose 16-bit storage scales). */
int ofd_field_absmax(ofd_handle *h, int level, double out[9]);

/* Stream of the handle (cudaStream_t) for callers that interleave work. */
void *ofd_stream(ofd_handle *h);

/* Device pointer + layout of one field level:  element (x, y, z) of the level
 * is at base[(x*dim2 + y)*pitch + z] in units of the storage type. */
typedef struct ofd_field_view {
    void *base;
    long pitch;      /* elements between consecutive y rows */
    int storage;
    float scale;
} ofd_field_view;
int ofd_field_view_get(ofd_handle *h, int field, int level, ofd_field_view *out);

/* Allocation-free FP64 sum of squares of one field (no counterpart in the
 * reference).  For callers that cannot allocate device memory: code running
 * during CUDA graph capture, plugins confined to another framework's memory
 * pool, and latency-bound serving loops that must not synchronise on the
 * allocator.  field: device array in the reference layout
 * float[dims[0]][dims[1]][dims[2]]; the sum covers the interior
 * [margin, dims-margin)^3; *out (device memory) receives the sum.  Work is
 * queued on stream (a cudaStream_t, NULL for the default stream).  Partial
 * sums live in a fixed 32 KB device array of the library, one entry per x
 * plane: at most 4096 interior planes (and at most 2^31 - 1 interior points
 * per plane), larger grids are rejected.  A call outside stream capture looks
 * up that array's device address in the current CUDA context and records it;
 * a call on a capturing stream uses the recorded address, so the first call
 * in each context (again after cudaDeviceReset) must come before any stream
 * capture.  All calls share the array: calls whose work overlaps on the GPU
 * race and must be serialised.  ofd_noalloc_last_error() describes
 * the last failure of this entry point on the calling thread. */
int ofd_sumsq_field_noalloc(const float *field, const int dims[3], int margin, double *out, void *stream);
const char *ofd_noalloc_last_error(void);

/* ------------------------------------------------------------------------
 * Regular-grid (acoustic) scheme: one field, three time levels, the update
 *
 *     u[t+1](x,y,z) = sum_k coef[k] * u[t - 1 + level[k]](x+dx, y+dy, z+dz)
 *
 * that RegularGrid emits for a second-order-in-time equation
 * (opesci/regulargrid.py:592-619 simple_kernel/kernel_sympy, time loop of
 * opesci/templates/regular3d_tmpl.py:94-105, level rotation
 * regulargrid.py:408-433).  Replaces the OpenMP time loop of that program.
 *
 * Terms are evaluated in the order given, as a left-to-right sum of
 * products rounded in the storage type (acc = c0*v0; acc = acc + ck*vk; no
 * fused multiply-add), which is how the reference's C expression
 * "c0*u[..] + c1*u[..] - ..." rounds.  Coefficients are the values of the
 * C literals (float literals, also in FP64 storage).  Offsets are bounded by
 * the margin on every axis.  The handle counts steps ti: step ti writes level
 * (ti%3 + 2)%3 from levels ti%3 (t-1) and (ti%3 + 1)%3 (t); margins are never
 * written.  Host arrays use the layout real_t[dim1][dim2][dim3].
 * ------------------------------------------------------------------------ */
#define OFD_REGULAR_MAX_TERMS 96

typedef struct ofd_regular_config {
    int dim[3];          /* dim1, dim2, dim3 = interior points + 2*margin */
    int margin;          /* space_order/2; the interior is [margin, dim-margin) */
    int storage;         /* OFD_F32 or OFD_F64 */
    int nterms;          /* 1..OFD_REGULAR_MAX_TERMS */
    int level[OFD_REGULAR_MAX_TERMS];      /* 1: level t, 0: level t-1 */
    int offset[OFD_REGULAR_MAX_TERMS][3];  /* dx, dy, dz, each in [-margin, margin] */
    double coef[OFD_REGULAR_MAX_TERMS];    /* exact value of the C literal */
    int variant;         /* 0: direct sweep (default), 1: shared-memory ring sweep */
} ofd_regular_config;

typedef struct ofd_regular ofd_regular;

/* three zeroed levels on the current device */
int ofd_regular_create(const ofd_regular_config *cfg, ofd_regular **out);
int ofd_regular_destroy(ofd_regular *h);
/* one level, host or device array of real_t[dim1][dim2][dim3] */
int ofd_regular_upload(ofd_regular *h, int level, const void *host);
int ofd_regular_download(ofd_regular *h, int level, void *host);
int ofd_regular_upload_device(ofd_regular *h, int level, const void *dev);
int ofd_regular_download_device(ofd_regular *h, int level, void *dev);
/* queue nsteps updates (one kernel each) on the handle's stream */
int ofd_regular_step(ofd_regular *h, int nsteps);
/* as ofd_regular_step, timed by CUDA events on the handle's stream; waits */
int ofd_regular_step_timed(ofd_regular *h, int nsteps, double *ms);
int ofd_regular_get_step(ofd_regular *h, long *steps);
int ofd_regular_set_step(ofd_regular *h, long steps);
int ofd_regular_sync(ofd_regular *h);
void *ofd_regular_stream(ofd_regular *h);

#ifdef __cplusplus
}
#endif
#endif /* OFD_H */

/*
 * faces_gb300.h -- C ABI of the GB300 (sm_103a) Faces halo-sum library.
 *
 * One context replaces the reference's per-rank `Faces` object
 * (gpu/v-26-messages/Faces.h:6-39) for all lx*ly*lz ranks at once: the MPI
 * rank grid becomes lx*ly*lz virtual ranks held in one device allocation,
 * rank-major.  Each rank's part uses the reference's DArray<double,6> layout
 * (gpu/DArray.h:34-38,91-101):
 *     idx = ix + n*iy + n^2*iz + n^3*jx + n^3*mx*jy + S4*jz,
 *     S4  = ceil(n^3*mx*my/512)*512,     rank stride = S4*mz.
 *
 * One share makes every point shared by 2 (face), 4 (edge) or 8 (corner)
 * element copies -- inside a rank and across its 26 neighbour ranks -- equal
 * to the FP64 sum of its copies.  The sum is formed as a tree in dimension
 * order (x pairs, then y pairs, then z pairs), the order of the reference's
 * Mugs oracle (gpu/Mugs.cc:140-202).
 *
 * Conventions: every call returns FACES_OK (0) or a negative FACES_E* code
 * and records a message for faces_last_error(); no exception crosses the ABI.
 * Device pointers must be 16-byte aligned (cudaMalloc gives 256).  `stream`
 * is a cudaStream_t (NULL: the legacy default stream).  Calls that take a
 * stream only enqueue work on it unless stated otherwise.  A context may be
 * used by one host thread at a time.
 */
#ifndef FACES_GB300_H
#define FACES_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FACES_OK 0
#define FACES_EINVAL (-1)       /* bad argument */
#define FACES_ECUDA (-2)        /* a CUDA call failed */
#define FACES_ENOMEM (-3)       /* device or host allocation failed */
#define FACES_EALIGN (-4)       /* pointer not 16-byte aligned */
#define FACES_EUNSUPPORTED (-5) /* combination not implemented */

/* faces_create flags */
#define FACES_PERIODIC 0x1u /* neighbours wrap around the rank grid; the
                               reference has none (MPI_PROC_NULL outside,
                               gpu/v-26-messages/Faces.cc:92-103) */
#define FACES_MESSAGES 0x2u /* v-26 strategy: every rank packs its 26 boundary
                               messages, the buffers are swapped by direction,
                               each rank unpack-adds its own copies.  Without
                               it one owner sums each shared point across
                               ranks in place (same values, no messages).  A
                               field with no neighbour rank (one non-periodic
                               rank) has no message: it takes the direct
                               step. */
#define FACES_GATHER 0x4u   /* force the generic one-thread-per-point kernel */
#define FACES_ROWS 0x8u     /* use the register row kernel instead of the
                               shared-memory tile kernel */
#define FACES_GENERAL 0x10u /* use the general tile step everywhere instead of
                               the periodic step (periodic direct-mode fields)
                               or the mixed step (the others: periodic step
                               on interior tiles); same result */
#define FACES_V6 0x20u      /* v-6 strategy (gpu/v-6-messages-basic/Faces.cc:
                               65-173): six face messages per rank, sweeps z,
                               then y, then x; each point gets the tree sum in
                               the order z, y, x pairs (equal to the other
                               modes on integer inputs, within the reference's
                               1e-15 check otherwise).  compute = 0 sums only
                               subdomain-boundary points (the reference's v-6
                               ignores compute). */
#define FACES_V6F 0x40u     /* v-6 in the fused form of gpu/v-6-messages-
                               overlap-fusable/Faces.cc:65-352: each sweep's
                               threads pack the later sweeps' messages for the
                               points they finish, the points no sweep changes
                               are packed up front; four launches per share
                               instead of six, the same messages and sums as
                               FACES_V6 bit for bit.  Not with FACES_V6 or
                               FACES_MESSAGES. */
#define FACES_SEAMS 0x80u   /* use the seam kernel: one thread per shared
                               point of each element's lower seam planes
                               (the point-per-thread form of gpu/v-26-
                               messages/Faces.cc:301-343), no shared memory;
                               direct mode only (not with FACES_MESSAGES,
                               FACES_V6 or FACES_V6F).  Without it the seam
                               kernel is still the default for direct-mode
                               fields with n >= 11 (FACES_ROWS and
                               FACES_GENERAL keep theirs). */
#define FACES_PACK_FUSED 0x100u /* message mode: the pack in the tile
                               kernel's prologue, one cooperative launch
                               per share (FUSE_SEND/FUSE_INNER of gpu/v-26-
                               messages/Faces.cc:175-239,301-343 on one
                               device): each block packs its share of the
                               pack's blocks, tiles that read a message or
                               write a subdomain-boundary point wait until
                               every block has, interior tiles run beside
                               the packing.  Same results; measured about
                               2% slower than the default (the pack as its
                               own launch, then the tile step) on a 3x3x3
                               grid of 16^3 n=6 ranks. */

typedef struct faces_ctx faces_ctx;

/* Faces::Faces(rank,lx,ly,lz,mx,my,mz,n) for every rank at once
 * (gpu/v-26-messages/Faces.cc:10-82): neighbour tables, message buffers. */
int faces_create(faces_ctx **ctx, int lx, int ly, int lz, int mx, int my, int mz, int n, unsigned flags);

/* Faces::~Faces (gpu/v-26-messages/Faces.cc:84-90).  NULL is accepted. */
int faces_destroy(faces_ctx *ctx);

/* DArray<double,6> strides of one rank (gpu/DArray.h:34-38; stride of ix is
 * 1, strides[0..5] are those of ix, iy, iz, jx, jy, jz), the doubles per rank
 * and in the whole field.  Any pointer may be NULL. */
int faces_layout(const faces_ctx *ctx, long strides[6], long *rank_doubles, long *total_doubles);

/* DArray's allocation (gpu/DArray.h:77-82): a zero-filled device field for
 * all ranks.  Free with faces_field_free. */
int faces_field_alloc(const faces_ctx *ctx, double **u);
int faces_field_free(double *u);

/* Faces::share(u, compute) (gpu/v-26-messages/Faces.h:18,
 * gpu/v-26-messages/Faces.cc:111-678) on every rank.  compute = 0 is the
 * reference's "shares without compute kernels" (gpu/main.cc:157-161): only
 * points on a subdomain boundary are summed.  Stream-ordered: returns once
 * the work is enqueued (the reference's share returns after completion;
 * synchronize the stream for that). */
int faces_share(faces_ctx *ctx, double *u, int compute, void *stream);

/* nshares consecutive shares (the `ni` loop of gpu/main.cc:180). */
int faces_share_n(faces_ctx *ctx, double *u, int compute, int nshares, void *stream);

/* gpu/main.cc:10-19: u(ix,iy,iz,jx,jy,jz) = jz*1e4 + jy*100 + jx + iz*0.01 +
 * iy*1e-4 + ix*1e-6 on every rank, each product and sum rounded once;
 * padding zero. */
int faces_init_ref(faces_ctx *ctx, double *u, void *stream);

/* integer-valued doubles uniform in [0,2^20): the top 20 bits of
 * splitmix64(seed*0x9E3779B97F4A7C15 + linear index); padding zero. */
int faces_init_int(faces_ctx *ctx, double *u, unsigned long long seed, void *stream);

/* The correctness check of gpu/main.cc:39-105 without a host copy: compares
 * u, after `nshares` shares (compute as given) of the initial state `init`
 * (0: faces_init_ref, 1: faces_init_int with `seed`), with the closed form
 * (every copy of a point with k seam axes holds S*2^(k*(s-1)), S the tree
 * sum of its initial copies).  Outputs (each may be NULL): rank_maxrel[nranks]
 * the per-rank maximum relative error |u-v|/(|u|+|v|); *npass the ranks
 * below 1e-15; where[7] = rank, ix, iy, iz, jx, jy, jz of the largest error
 * and vals[2] = (u, expected) there.  Beyond the reference's rule, the page
 * padding of each jz slab must still hold the zeros both inits write: a
 * nonzero padding double counts as relative error 1 (NaN anywhere: infinite),
 * and where it is the largest error, where[] = rank, -1 x 5, jz.
 * Synchronous. */
int faces_check(faces_ctx *ctx, const double *u, int init, unsigned long long seed, int nshares, int compute,
                double *rank_maxrel, double *maxrel, int *npass, int where[7], double vals[2], void *stream);

/* End-to-end call for host data: copies u_in (host, total doubles) to the
 * context's device field, runs nshares shares, copies the result to u_out
 * (host; may equal u_in).  Synchronous.  Pinned host memory is fastest. */
int faces_run_host(faces_ctx *ctx, const double *u_in, double *u_out, int compute, int nshares, void *stream);

/* faces_run_host for njobs independent fields of this context's shape: job j
 * uploads u_in[j], runs nshares shares and downloads to u_out[j].  Three
 * device fields and two copy streams let job j+1's upload and job j-1's
 * download run while job j's shares run on a third stream of the context
 * (the third field: an upload waits for the download of the job three
 * before it, two jobs' shares of slack); all three streams start
 * after the work already on `stream`, and `stream` ends after them (any
 * stream works, the legacy default one included).  u_out[j] may equal u_in[j], and
 * outputs may repeat across jobs (downloads run in job order); an input may
 * not be an earlier job's output (FACES_EINVAL), and buffers must not overlap
 * otherwise.  Synchronous; the overlap needs pinned host memory.
 * No counterpart in the reference, whose main loop holds one field per
 * process (gpu/main.cc:169-184). */
int faces_run_host_many(faces_ctx *ctx, int njobs, const double *const *u_in, double *const *u_out, int compute,
                        int nshares, void *stream);

/* Work decomposition: elements per x-chunk (<= 0: default; the tile kernel
 * rounds down to a power of 2, at most 8, or 16/32 for n <= 5/3), width (<= 0: default): tiles per thread
 * block for the row kernel, resident blocks per SM for the tile kernel, and
 * the tile kernel's order (< 0: default = 2, 0: blocks stride over the tiles,
 * 1: each block takes a contiguous range of x-chunks, 2 + 16*u: blocks stride
 * over units of u consecutive x-chunks of a column, listed chunk group first,
 * u = 0 half a column; 3: periodic step only, one warp per tile instead of
 * one block, no block barriers).  With the seam kernel (FACES_SEAMS, and
 * the default for direct-mode fields with n >= 11): elements per x-chunk of
 * its chunked form, resident blocks per SM, and the form (order 0 chunked,
 * 1 lean: one thread per face slot of every element, plus a launch for the
 * open boundary planes; < 0: lean where the field gives four waves of
 * threads).  Returns to the default kernel. */
int faces_set_tuning(faces_ctx *ctx, int chunk, int width, int order);

/* Times the tile step on the field u over elements per tile (default, half,
 * double), units (half a column, one chunk, warp tiles) and resident blocks
 * per SM (default, 2), the general tile step and the row kernel at their
 * defaults, and in direct mode the seam kernel (chunked at its default and
 * at a longer chunk; lean), each after one warm-up over at least `trials`
 * shares and at least about 1 ms of shares, and keeps the fastest
 * (faces_set_tuning's settings and the kernel; faces_set_tuning returns to
 * the default kernel).  Every timed launch is a share of
 * u: returns how many it applied (>= 0; re-initialise u afterwards) or an
 * error code.  The reference fixes these choices at compile time
 * (MAXTHREADS, gpu/gpu.h:185-200).  Synchronous. */
int faces_autotune(faces_ctx *ctx, double *u, int compute, int trials, void *stream);

/* The tile step's current settings: elements per tile, x-chunks per unit
 * of work, blocks launched, the kernel (0 the tile step, 1 the general tile
 * step, 2 the row kernel, 3 the seam kernel) and the tile order (as
 * faces_set_tuning; 3 warp tiles; seam kernel: 0 chunked, 1 lean).  Any
 * pointer may be NULL. */
int faces_get_tuning(const faces_ctx *ctx, int *chunk, int *unit_chunks, int *blocks, int *kernel, int *order);

/* The device-side status bits of the fused message-mode step
 * (FACES_PACK_FUSED), read and cleared (synchronous): bit 0 = a block's wait
 * for the others' packing ran out (bounded, about a second; the shares since
 * the last call are then not to be trusted).  0 when all is well. */
int faces_status(faces_ctx *ctx, int *bits);

/* Test hook for the fused step's bounded wait: with extra = 1 every block
 * that waits waits for one more arrival than the launch has, so each such
 * wait runs out after `polls` polls (of about 64 ns or more) and sets status
 * bit 0 instead of hanging; extra = 0, polls = 4194304 are the defaults
 * (about a second).  The shares run with extra = 1 are wrong; the context
 * stays usable. */
int faces_test_pack_wait(faces_ctx *ctx, int extra, long polls);

/* Kernel launches one share enqueues with the current settings. */
int faces_launches_per_share(const faces_ctx *ctx, int compute);

/* Message of the last failed call on this thread ("" if none). */
const char *faces_last_error(void);

/* Doubles in the device array faces_share_static works in (32 MiB). */
#define FACES_STATIC_SCRATCH_DOUBLES (4L << 20)

/* One message-mode share (FACES_MESSAGES) of the field u -- lx*ly*lz ranks of
 * mx*my*mz elements of n^3 points in the layout above -- that allocates no
 * device memory.  No counterpart in the reference: it exists for callers that
 * cannot call cudaMalloc, such as applications that give all device memory
 * to their own pool at start-up, and latency-critical loops that cannot take
 * the device-wide synchronisation cudaMalloc and cudaFree imply.  Its working
 * memory (neighbour table, message offsets, the 26 messages of every rank)
 * lives in one file-scope device array of FACES_STATIC_SCRATCH_DOUBLES
 * doubles, held by every GPU that loads the library until the process
 * exits; a field whose tables and messages do not fit is rejected with
 * FACES_EINVAL.  The array's device address is taken on the first call on
 * each device, so make that first call before any stream capture; it is kept
 * until the process exits, so a device reset (cudaDeviceReset) voids it and
 * the entry point must not be called on that device again.  Each device has
 * its own array; all calls on one device share it and each rewrites what it
 * reads, so calls that overlap on the same device (two unordered streams)
 * race.  flags: FACES_PERIODIC or 0.  Stream-ordered like faces_share; the
 * result equals faces_share with FACES_MESSAGES bit for bit. */
int faces_share_static(double *u, int lx, int ly, int lz, int mx, int my, int mz, int n, unsigned flags,
                       int compute, void *stream);

/* ---- Batches: many independent fields advanced together ----
 *
 * The reference advances one field per process: a Faces object per field
 * and one share call per step (gpu/main.cc:169-180).  A batch holds any
 * number of fields of different shapes on one GPU; faces_batch_share
 * advances all of them by one share, bit for bit as faces_share would, with
 * one launch of a persistent kernel for the fields it takes (direct mode,
 * 2 <= n <= 10, compute = 1) and one faces_share per other field. */
typedef struct faces_batch faces_batch;

int faces_batch_create(faces_batch **b);

/* Adds the field u (device, 16-byte aligned, laid out as for faces_create
 * with these arguments) and returns its index in *field_id (may be NULL).
 * Only before faces_batch_commit. */
int faces_batch_add(faces_batch *b, double *u, int lx, int ly, int lz, int mx, int my, int mz, int n,
                    unsigned flags, int *field_id);

/* Builds the device work list; the batch is fixed afterwards. */
int faces_batch_commit(faces_batch *b);

/* One share of every field: one batched launch plus one faces_share per
 * field the batched kernel does not take.  Stream-ordered. */
int faces_batch_share(faces_batch *b, int compute, void *stream);

/* nshares shares of every field as one CUDA graph, captured on the first
 * call for each (nshares, compute) and replayed after.  Stream-ordered. */
int faces_batch_share_n(faces_batch *b, int compute, int nshares, void *stream);

/* One share of every field, one faces_share call per field (the reference's
 * pattern; the baseline the batched launch is measured against). */
int faces_batch_share_each(faces_batch *b, int compute, void *stream);

/* Work list settings: unit_div (units are 1/unit_div of a column's
 * x-chunks; <= 0 keeps it), resident blocks per SM (<= 0 keeps it), half
 * (stage size: 0 default, ~20 KB; 1 half-size stages, which keep 4 blocks
 * per SM; 2 stages of up to ~28 KB, 2 blocks per SM; 1 and 2 only when every
 * batched field is periodic and in direct mode; < 0 keeps it -- periodic-step
 * tiles take as many elements as the stage holds), run
 * (units a block takes in a row before striding by the grid; <= 0 keeps it). */
int faces_batch_tune(faces_batch *b, int unit_div, int blocks_per_sm, int half, int run);

/* The warp form of the batched launch (every batched field periodic, stage
 * form 0 or 2): fields with n <= max_n (at most 5; 0: none; < 0 keeps it)
 * are cut into whole-column units that the first blocks of the launch take
 * warp by warp -- each warp stages, sums and stores its own tiles, with no
 * block barrier -- while the other blocks run the block pipeline over the
 * rest; those first blocks are `boost` (<= 0 keeps it) times the small
 * fields' share of the points, of all blocks.  Default: max_n 5, boost 2. */
int faces_batch_tune_warp(faces_batch *b, int max_n, int boost);

/* The warp form's max_n and boost, its units and its blocks (each may be
 * NULL). */
int faces_batch_warp_info(const faces_batch *b, int *max_n, int *boost, int *warp_units, int *warp_blocks);

/* Times the batched launch over unit_div in {1,2,4,8,64}, the tile lengths
 * (when allowed), runs of 1 or 8 units per block and the resident blocks per SM that fit, `trials` launches each (after one warm-up), and
 * keeps the fastest; then, with those, the warp form's max_n in {0,3,4,5}
 * and boost in {1,2,3,4}.  Every launch is a share of the fields in the batched
 * launch (the others are untouched): returns how many shares it applied to
 * each of them (>= 0), or a negative error code.  Synchronous. */
int faces_batch_autotune(faces_batch *b, int trials, void *stream);

/* fields, fields in the batched launch, work units, unit_div, blocks of the
 * batched launch, tile length form, units a block takes in a row (each may
 * be NULL). */
int faces_batch_info(const faces_batch *b, int *fields, int *fused_fields, int *units, int *unit_div, int *blocks,
                     int *half, int *run);

int faces_batch_destroy(faces_batch *b);

/* ---- Job server: halo-sum jobs arriving over time ----
 *
 * The reference runs one job per launch of its executable (gpu/main.cc:134-
 * 197: one field, nk*nj*ni shares, then exit).  A server keeps many jobs of
 * different sizes resident on one GPU: each job is admitted, in arrival
 * order, when its field fits the HBM budget (and the job limit); from then
 * on every running job takes one share per tick, all of them in one
 * persistent launch (continuous batching: jobs that arrive while others run
 * join at the next tick, finished ones leave).  A job's result is bit for
 * bit the field faces_share_n gives it alone.  Jobs run in direct mode with
 * 2 <= n <= 10.  One host thread at a time may call a server. */
typedef struct faces_server faces_server;

typedef struct faces_job {
  int lx, ly, lz, mx, my, mz, n; /* as faces_create */
  unsigned flags;                /* FACES_PERIODIC or 0 */
  int nshares;                   /* shares to run (nk*nj*ni), >= 1 */
  int init;                      /* 0: faces_init_ref, 1: faces_init_int(seed), 2: copy host_in */
  unsigned long long seed;
  const double *host_in;         /* init = 2: the field (total doubles), read during admission */
} faces_job;

typedef struct faces_serve_stats {
  long long submitted, admitted, completed;
  long long ticks;      /* scheduling rounds, each one share of every running job */
  long long launches;   /* kernel launches (steps and initialisations) */
  long long job_shares; /* shares run, summed over jobs */
  double point_shares;  /* points times shares, summed over jobs */
  size_t resident_bytes, peak_resident_bytes, budget_bytes;
  int queued, running;
} faces_serve_stats;

#define FACES_SERVE_PLAIN 0x1u        /* one single-field launch per running job per tick (the plain form) */
#define FACES_SERVE_RELEASE_DONE 0x2u /* free a job's field as soon as it is done */

/* A server with an HBM budget for job fields (bytes) and a limit on running
 * jobs (<= 0: none).  Its memory comes from a stream-ordered pool that keeps
 * what it has taken until faces_server_destroy. */
int faces_server_create(faces_server **s, size_t budget_bytes, int max_jobs, unsigned flags);

/* Queues a job (arrival = now); rejected if its field alone exceeds the
 * budget.  *job_id identifies it afterwards. */
int faces_server_submit(faces_server *s, const faces_job *job, long long *job_id);

/* One scheduling round: retire finished ticks, admit, launch the next tick.
 * wait != 0: when no launch is possible, block until the oldest tick
 * finishes.  Returns the jobs that became done (>= 0) or an error code;
 * FACES_ENOMEM when a queued job can never be admitted because done jobs
 * that were not released hold the budget. */
int faces_server_poll(faces_server *s, int wait);

/* Polls until every submitted job is done; returns the jobs that became done. */
int faces_server_drain(faces_server *s);

/* state: 0 queued, 1 running, 2 done, 3 released; shares done; seconds from
 * arrival to admission (wait_s) and to the GPU completion of its last share
 * (latency_s), -1 while not reached.  Any pointer may be NULL. */
int faces_server_job_status(faces_server *s, long long job_id, int *state, int *shares_done, double *wait_s,
                            double *latency_s);

/* Device field of a running or done job and its size in doubles. */
int faces_server_field(faces_server *s, long long job_id, double **u, long *total_doubles);

/* Copies a done job's field to host memory (synchronous). */
int faces_server_fetch(faces_server *s, long long job_id, double *host_out);

/* Frees a done job's field and forgets the job. */
int faces_server_release(faces_server *s, long long job_id);

int faces_server_stats(const faces_server *s, faces_serve_stats *st);

/* Work list settings of the batched launch (as faces_batch_tune): unit_div
 * (units are 1/unit_div of a column's x-chunks; default 1, whole columns),
 * run (units a block takes in a row; default 1), half (tile form 0, 1 or 2;
 * used for ticks in which every running job is periodic, else 0).
 * Values <= 0 (half < 0) keep the setting. */
int faces_server_tune(faces_server *s, int unit_div, int run, int half);

/* The warp form of the server's batched launch, as faces_batch_tune_warp:
 * jobs with n <= max_n (at most 5; 0: none; < 0 keeps it) are taken warp by
 * warp by the first blocks, `boost` (<= 0 keeps it) times their share of the
 * points.  Default: max_n 5, boost 2.  Applies from the next tick. */
int faces_server_tune_warp(faces_server *s, int max_n, int boost);

/* Replays an arrival trace in real time: job i is submitted when
 * arrival_s[i] seconds (non-decreasing) have passed since the call began,
 * stamped with that time, and the call returns when all are done.
 * job_ids[i], latency_s[i] (arrival to completion) and *makespan_s may be
 * NULL. */
int faces_server_run_trace(faces_server *s, int njobs, const faces_job *jobs, const double *arrival_s,
                           long long *job_ids, double *latency_s, double *makespan_s);

/* Waits for the server's work and frees everything it holds.  NULL is
 * accepted. */
int faces_server_destroy(faces_server *s);

#ifdef __cplusplus
}
#endif

#endif /* FACES_GB300_H */

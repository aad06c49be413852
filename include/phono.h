/*
 * phono.h - C ABI of libphono_gpu.so, the GB300 (sm_103a) elastic FDTD
 * solver that stands in for phonomena's time-stepping solver.
 *
 * The reference solver is the Python class BaseSolver
 * (phonomena/simulation/base_solver.py:172-571) behind the plugin interface
 * found by common.importSolver / findSolvers (phonomena/common.py:88-110).
 * A plugin module (phonomena_gb300/solver_gb300.py) binds these entry points
 * with ctypes; each declaration names the reference code it replaces.
 *
 * Conventions
 *  - Plain C types only; host pointers unless a name says "dev".
 *  - Every call returns PHONO_OK (0) or a negative PHONO_ERR_* code and
 *    never aborts; phono_last_error() gives a message for the calling thread.
 *  - A handle owns its device memory and one CUDA stream; calls on a handle
 *    are ordered on that stream.  Use one handle per host thread.
 *  - Arrays are C order with x slowest, in the reference shapes
 *    (phonomena/simulation/grid.py:88-110): ux (nx-1, ny, nz),
 *    uy (nx, ny-1, nz), uz (nx, ny, nz-1); nx, ny, nz are mesh NODE counts
 *    (Grid.x.size, ...), each >= 3.
 */
#ifndef PHONO_H
#define PHONO_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PHONO_ABI_VERSION 2

#define PHONO_OK 0
#define PHONO_ERR_ARG (-1)      /* invalid argument */
#define PHONO_ERR_CUDA (-2)     /* CUDA runtime error */
#define PHONO_ERR_NOMEM (-3)    /* device or host allocation failed / over budget */
#define PHONO_ERR_STATE (-4)    /* call not valid in the current state */
#define PHONO_ERR_NUMERIC (-5)  /* non-finite value seen in the recorded surface */
#define PHONO_ERR_TIMEOUT (-6)  /* a bounded device wait ran out; the state of that step is invalid */

/* arithmetic scheme */
#define PHONO_F64 0  /* reference leapfrog in the reference's op order, bit-identical results
                      * (divisions by the mesh spacings through a table of double-word
                      * reciprocals, which gives the IEEE quotients) */
#define PHONO_F32K 1 /* FP32 velocity form, Kahan-compensated displacement */
#define PHONO_F64V 2 /* the F32K scheme in FP64: fast FP64 reference for error figures */

/* z = 0 displacement row (base_solver.py:511-516) */
#define PHONO_SURFACE_REFERENCE 0 /* precedence as written at :516 */
#define PHONO_SURFACE_CORRECTED 1 /* (T3[...,1] - T3[...,0]) / fdz */

/* the four walls x=N, y=0, y=N, z=N (base_solver.py:519-554) */
#define PHONO_BC_ABSORBING 0 /* first-order absorbing faces, reference order */
#define PHONO_BC_RIGID 1     /* u = 0 on those faces */

/* source overwrite (base_solver.py:251) */
#define PHONO_SOURCE_LINE 0 /* uz[0, :, 0] = s(tt) (reference) */
#define PHONO_SOURCE_WALL 1 /* uz[0, :, :] = s(tt) */

/* fields for phono_download / phono_upload */
#define PHONO_FIELD_UX 0
#define PHONO_FIELD_UY 1
#define PHONO_FIELD_UZ 2
#define PHONO_FIELD_UX_OLD 3 /* F64: u at the previous step */
#define PHONO_FIELD_UY_OLD 4
#define PHONO_FIELD_UZ_OLD 5
#define PHONO_FIELD_VX 6 /* F32K, F64V: velocity at the last half step */
#define PHONO_FIELD_VY 7
#define PHONO_FIELD_VZ 8
#define PHONO_FIELD_CX 9 /* F32K, F64V: Kahan compensation */
#define PHONO_FIELD_CY 10
#define PHONO_FIELD_CZ 11

/* Material table row: C00 C01 C02 C10 C11 C12 C20 C21 C22 C33 C44 C55 rho.
 * Replaces the per-node Material.C (nx,ny,nz,6,6) and Material.P arrays
 * (phonomena/simulation/material.py:48-63) by one row per material id. */
#define PHONO_TABLE_COLS 13

typedef struct phono_desc {
  int nx, ny, nz;                /* mesh nodes per axis, each >= 3 */
  const double *fdx, *fdy, *fdz; /* full spacings, n-1 values (SI)  grid.py:117-120 */
  const double *sdx, *sdy, *sdz; /* staggered spacings, n-2 values  grid.py:122-127 */
  const uint8_t *mat;            /* nx*ny*nz node material ids */
  const double *table;           /* nmat rows of PHONO_TABLE_COLS */
  int nmat;                      /* 1..256 */
  double dt;                     /* time step (Material.dt, material.py:80-93) */
  int precision;                 /* PHONO_F64 | PHONO_F32K | PHONO_F64V */
  int surface_mode;              /* PHONO_SURFACE_* */
  int bc;                        /* PHONO_BC_* */
  int source_mode;               /* PHONO_SOURCE_* */
  int max_steps;                 /* capacity: source samples and surface records */
  int record_every;              /* record uz[:, :, 0] after every k-th step; 0 = off */
  int tile_j;                    /* tile height along y: 4, 8 or 16; 0 = default (F32K 4, else 8) */
  int x_segment;                 /* planes per block segment; -L: L-plane segments, the last 2L planes in four shorter ones; 0 = default (24) */
} phono_desc;

typedef struct phono_handle phono_handle;

/* Device bytes phono_create would allocate for a mesh of nx*ny*nz nodes with
 * these settings (each allocation rounded up to 512 bytes): what a caller
 * admitting simulations against a memory budget charges per handle.  No
 * reference counterpart. */
int phono_footprint(int nx, int ny, int nz, int precision, int max_steps, int record_every, size_t *bytes);

/* Allocate the device state (zero fields) for one simulation.
 * Replaces BaseSolver.init (base_solver.py:194-222). */
int phono_create(const phono_desc *desc, phono_handle **out);

/* Source sample s(tt) of every global step tt < n (n <= max_steps): the value
 * the reference writes into uz[0,:,0] before step tt (base_solver.py:251),
 * from update_sin / update_ricker (base_solver.py:294-312). */
int phono_set_source(phono_handle *h, const double *samples, int n);

/* Advance nsteps time steps; per step a tile launch and a face launch (one
 * launch when ny == 3), replayed from captured CUDA graphs of 12 steps.  Replaces the loop body of BaseSolver.run
 * (base_solver.py:245-266): source, update_T, update_T_BC, update_u,
 * update_u_BC, time_step.  Asynchronous on the handle's stream. */
int phono_step(phono_handle *h, int nsteps);

/* Advance nsteps time steps like phono_step, but without the graph and with
 * a CUDA event before and after each launch, so that the two kernels of a
 * step are timed apart: *tile_ms = the summed device time of the tile
 * launches (the fused launch when ny == 3), *face_ms = that of the face
 * launches.  Blocks until done.  Results are those of phono_step.  No
 * reference counterpart (measurement). */
int phono_time_kernels(phono_handle *h, int nsteps, float *tile_ms, float *face_ms);

/* Global steps completed so far (host-side count of enqueued steps). */
int phono_steps_done(const phono_handle *h);

/* Zero the state, the surface records and the step counter: the handle is
 * as after phono_create (material, spacing and source kept).  Stands in for
 * the field allocation of Grid.update (grid.py:87-110) on a re-run. */
int phono_reset(phono_handle *h);

/* Replace the material ids and table of a handle (same mesh shape): a new
 * crystal in an existing slot.  Replaces Material.setConstants
 * (material.py:55-63) on the device. */
int phono_set_materials(phono_handle *h, const uint8_t *mat, const double *table, int nmat);

/* Material ids of a phononic crystal built on the device: a square lattice
 * (pitch `pitch` cells, ncx x ncy cells, cell (p, q) covering nodes
 * [p*pitch, (p+1)*pitch) in x and y, the last cell also the rest) of vertical
 * cylindrical holes centred in their cells, from z = 0 down through node
 * `depth`.  A node is inside the hole of its cell when its squared distance
 * from the centre is below the squared radius (FP64).  Inside: the cell's id;
 * elsewhere: `host`.  The table as in phono_set_materials.  Replaces the
 * reference's per-node fill of the inclusion nodes (material.py:59-63,
 * grid.py:158-175) with one kernel.  No reference counterpart as a call. */
typedef struct phono_lattice {
  int pitch;             /* lattice pitch in cells */
  int ncx, ncy;          /* lattice cells along x and y */
  const double *radius;  /* ncx*ncy hole radii in cells, x slowest */
  const uint8_t *kind;   /* ncx*ncy material id inside each hole */
  int depth;             /* holes fill z = 0..depth (nodes) */
  int host;              /* material id outside the holes */
} phono_lattice;

int phono_set_lattice(phono_handle *h, const phono_lattice *lat, const double *table, int nmat);

/* Material ids of the reference's inclusion model, built on the device.
 * Replaces Material.setConstants (phonomena/simulation/material.py:55-63)
 * with the inclusion search of Grid.inclusionIndices
 * (phonomena/simulation/grid.py:158-175), on any mesh the reference builds
 * (non-uniform x and y included), without the per-node 6x6 C and P arrays.
 *
 * An inclusion is a vertical cylinder as Grid.targets holds it: centre
 * (tx, ty), radius tr and depth tz in mesh units, float32 (the reference's
 * trgt_dtype).  Node (i, j, k) lies in inclusion t when
 *   sqrt((x[i] - tx)^2 + (y[j] - ty)^2) < tr     (FP64, as NumPy computes it)
 * and k is in the inclusion's z selection.  The z selection reproduces the
 * reference exactly, including how grid.py:174 rebinds `z`: the first
 * inclusion keeps the nodes with z[k] <= tz; each later inclusion keeps the
 * node indices p < (the previous selection's length) with p <= tz.  Where
 * inclusions overlap, the later one in the list wins (the reference
 * overwrites in list order).  Every other node gets `host`.
 *
 * x, y, z are the node coordinates (Grid.x, Grid.y, Grid.z: nx, ny, nz
 * values, strictly ascending, host memory).  The table as in
 * phono_set_materials; the absorbing faces take their wave speeds from the
 * material that ends up at node (0, 0, 0). */
typedef struct phono_inclusions {
  const double *x, *y, *z;        /* node coordinates in mesh units */
  int n;                          /* inclusions (rows of Grid.targets), >= 0 */
  const float *tx, *ty, *tz, *tr; /* Grid.targets fields x, y, z, r */
  const uint8_t *id;              /* material id of each inclusion; NULL: all `inside` */
  int inside;                     /* id of every inclusion when id is NULL (the secondary material) */
  int host;                       /* id outside the inclusions (the primary material) */
} phono_inclusions;

int phono_set_inclusions(phono_handle *h, const phono_inclusions *inc, const double *table, int nmat);

/* Copy the handle's material ids (nx*ny*nz bytes, C order) to host, e.g. to
 * check a device-built crystal.  No reference counterpart (the reference's
 * Material.C / P are host arrays already). */
int phono_download_materials(phono_handle *h, uint8_t *host, size_t bytes);

/* The handle's cudaStream_t (as void*), for callers that record their own
 * CUDA events around phono_step. */
void *phono_stream(phono_handle *h);

/* Wait for the handle's stream; returns PHONO_ERR_TIMEOUT if a tile block's
 * bounded wait for its plane copies ran out (the block flagged it, waited for
 * the copies it had issued and returned; the state of that step is invalid
 * and phono_reset clears the flag), PHONO_ERR_NUMERIC if a recorded surface
 * value was not finite. */
int phono_sync(phono_handle *h);

/* Test hook for the time-out path above; no reference counterpart.  Every
 * mbarrier wait of the tile pass gives up after `polls` polls (0: the default
 * budget, about 0.3 s).  With skip_plane >= 0, every tile block that reads
 * plane skip_plane arms that plane's barrier but issues no copy for it, so
 * its wait on it runs out; the next phono_sync returns PHONO_ERR_TIMEOUT.
 * phono_test_wait_timeout(h, 0, -1) turns it off. */
int phono_test_wait_timeout(phono_handle *h, int polls, int skip_plane);

/* Copy surface records [first, first+count) to host: count * nx * ny values
 * (float for PHONO_F32K, double otherwise), record r = uz[:, :, 0]
 * after global step (r+1)*record_every - 1.  Stands in for the per-step
 * uz dataset of the reference writer (base_solver.py:114-116,153-155). */
int phono_read_surface(phono_handle *h, int first, int count, void *host_out);

/* Copy a field of the current state to / from host (reference shape, element
 * size 4 for PHONO_F32K, 8 otherwise).  Download of UX..UZ is what
 * the reference leaves in g.ux, g.uy, g.uz after run. */
int phono_download(phono_handle *h, int field, void *host, size_t bytes);
int phono_upload(phono_handle *h, int field, const void *host, size_t bytes);

/* Checkpoint / resume (no reference counterpart; for preempting and
 * restarting long runs).  A checkpoint is the state fields of the scheme
 * (F64: UX..UZ and UX_OLD..UZ_OLD; F32K / F64V: UX..UZ, VX..VZ, CX..CZ), the
 * step count and the surface records so far.  To resume into a handle made
 * with the same description and source: phono_set_steps_done first (it
 * selects the buffers the fields belong to), then phono_upload of each field
 * and phono_upload_surface of the records; the run then continues bit for
 * bit as if it had not stopped. */
int phono_set_steps_done(phono_handle *h, int steps);
int phono_upload_surface(phono_handle *h, int first, int count, const void *host_in);

/* Element size in bytes of the handle's fields (8 or 4). */
int phono_elem_size(const phono_handle *h);

/* Kinetic and strain energy of the current state, FP64 accumulation in a
 * fixed order (the same state gives the same bits): out[0] = sum rho v^2 / 2
 * over the interior displacement points, out[1] = sum T:e / 2 over the
 * reference's stress points, unit weights (no cell volume).  Blocks until
 * done.  No reference counterpart (error metric). */
int phono_energy(phono_handle *h, double out[2]);

/* Energy of a state held in the caller's own device buffers, computed
 * without allocating anything.  No counterpart in the reference.
 *
 * For callers that cannot call cudaMalloc/cudaFree: applications whose
 * device memory is owned by another allocator (a framework's caching pool, a
 * fixed reservation made at start-up) and latency-bound loops that must not
 * take the implicit device synchronisation of cudaFree.  The per-plane
 * partial sums go to a file-scope __device__ scratch array of
 * PHONO_ENERGY_STATIC_MAX_NX entries (128 KiB, held by every GPU that loads
 * the library until the process exits); nx above that limit is rejected
 * with PHONO_ERR_ARG.  All calls share that array: calls whose kernels
 * overlap on the GPU race on it and must be serialised by the caller (one
 * stream, or events).  Every call overwrites the partials it reads, so
 * nothing has to be cleared between calls.  The first call on a device
 * looks up the array's device address (cudaGetSymbolAddress) with that
 * device current.  The address is cached for the life of the device's
 * primary context: do not call this again on a device after
 * cudaDeviceReset.
 *
 * Inputs are dense arrays in the reference shapes, element type given by
 * `precision`, all device pointers; out_dev receives two doubles
 * (kinetic, strain) in device memory, written on `stream` (a cudaStream_t,
 * NULL for the default stream); the call does not synchronise.  Material
 * ids must be below nmat; the kernel checks every id before it reads the
 * table, and an id at or past nmat makes both outputs NaN (the table is
 * never read out of bounds). */
#define PHONO_ENERGY_STATIC_MAX_NX 8192

typedef struct phono_energy_dense {
  int nx, ny, nz;                /* mesh nodes, 3 <= nx <= PHONO_ENERGY_STATIC_MAX_NX */
  int precision;                 /* PHONO_F64: velocity from (u - u_old)/dt; F32K / F64V: v given */
  const void *ux, *uy, *uz;      /* displacement (float for F32K, double otherwise) */
  const void *vx, *vy, *vz;      /* F32K / F64V: velocity; F64: u at the previous step */
  const uint8_t *mat;            /* nx*ny*nz node material ids, each < nmat */
  const double *table;           /* nmat material rows of PHONO_TABLE_COLS doubles */
  const double *fdx, *fdy, *fdz; /* full spacings (n-1 values) */
  const double *sdx, *sdy, *sdz; /* staggered spacings (n-2 values) */
  double dt;
  int nmat;                      /* rows of table, 1..256 */
} phono_energy_dense;

int phono_energy_static(const phono_energy_dense *in, double *out_dev, void *stream);

/* Batches: many simulations stepped together.  In the default (persistent)
 * scheme every time step is one persistent tile launch (CTAs pull (instance,
 * tile) work items until none are left) and one face launch for all active
 * instances, replayed from a captured CUDA graph; phono_batch_set_mode
 * selects the other scheme.  The reference runs one simulation per solver
 * object (base_solver.py:245-266) and has no counterpart; the per-instance
 * arithmetic is that of phono_step, bit for bit.  Instances are handles made
 * by phono_create with the batch's precision and ny >= 4 (and the batch's
 * tile_j in the persistent scheme); each keeps its own x segments.  While a
 * handle is in a batch, phono_step, phono_reset, phono_set_materials,
 * phono_upload and phono_set_tiling on it return PHONO_ERR_STATE; call
 * phono_batch_sync before reading it.  A handle destroyed while in a batch
 * leaves the batch. */
typedef struct phono_batch phono_batch;

int phono_batch_create(int capacity, int precision, int tile_j, phono_batch **out);
/* Launch scheme of an empty batch (PHONO_ERR_STATE once it holds an
 * instance).  PHONO_BATCH_PERSISTENT (the default): the persistent tile
 * launch above, every instance at the batch's tile_j.  PHONO_BATCH_STREAMS:
 * every instance runs its own step kernels (those of phono_step, with its own
 * tile_j and x segments) on one of `streams` worker streams (1..256), so that
 * instances run side by side.  Each instance replays its own graph of 12
 * steps (captured when it joins) and starts its next chunk as soon as its
 * previous one is done; phono_batch_step returns once every worker's work is
 * queued and the batch stream waits for all of them.  Results are those of
 * phono_step in both schemes. */
#define PHONO_BATCH_PERSISTENT 0
#define PHONO_BATCH_STREAMS 1
int phono_batch_set_mode(phono_batch *b, int mode, int streams);
/* Attach h for nsteps more steps; returns the slot (>= 0) or an error code. */
int phono_batch_add(phono_batch *b, phono_handle *h, int nsteps);
int phono_batch_remove(phono_batch *b, int slot);
/* Steps an instance still has to take (0 when done). */
int phono_batch_remaining(const phono_batch *b, int slot);
/* Advance every active instance by up to nsteps (each stops at its budget). */
int phono_batch_step(phono_batch *b, int nsteps);
int phono_batch_sync(phono_batch *b);
int phono_batch_last_step_ms(phono_batch *b, float *ms);
void phono_batch_destroy(phono_batch *b);

/* Change the tile shape of a handle (0 keeps a value): tile_j rows per block
 * (4, 8, 16) and x_segment planes per block column (-L: tapered, as in
 * phono_desc; PHONO_ERR_ARG when that takes more than 64 segments).  Results
 * do not depend on the tile shape; the tuner (phonomena_gb300/autotune.py) calls this to
 * time candidates on one handle.  No reference counterpart. */
int phono_set_tiling(phono_handle *h, int tile_j, int x_segment);

/* Tile height (0 keeps it) and an explicit list of x segments: n lengths in
 * planes, dispatched in list order, each >= 1, adding up to nx - 1, n <= 64.
 * A block marches one segment of one (y, z) tile, so the list sets how the
 * launch's work is cut into blocks; long segments first and a shortening
 * tail keep the last wave of blocks short.  phono_set_tiling(h, tj, 0) keeps
 * the list.  Results do not depend on it.  No reference counterpart. */
#define PHONO_MAX_SEGMENTS 64
int phono_set_segments(phono_handle *h, int tile_j, const int *lengths, int n);

/* Device time of the last phono_step call in milliseconds (CUDA events). */
int phono_last_step_ms(phono_handle *h, float *ms);

void phono_destroy(phono_handle *h);

/* Message of the last failed call on this thread ("" if none). */
const char *phono_last_error(void);

int phono_abi_version(void);

#ifdef __cplusplus
}
#endif

#endif /* PHONO_H */

/*
 * tecs_gpu.h -- C ABI of the GB300 (sm_103a) cell-step library.
 *
 * The TECS reference exposes its hot path as C++ templates (Simulation,
 * pair finders, integrators, com fixers).  This header is the thin C layer
 * beneath those templates: plain pointers and sizes, no C++ or torch types,
 * so a ctypes / cffi / cgo / JNI stub can bind it directly.  Each entry point
 * names the reference interface it replaces.
 *
 * Conventions
 *   - Every function returns 0 on success and a negative status on failure;
 *     tecs_last_error() then holds a message for the calling thread.
 *   - "host" pointers are ordinary CPU memory (pinned or pageable); "device"
 *     pointers are CUDA global memory on the simulation's device.
 *   - Positions are AoS float[n][dims] (the byte layout of the reference's
 *     View<VectorN<float, dims>>); polarities are float[n][2] (theta, phi),
 *     the layout of View<Polarity_<float>>.
 *   - Work is queued on the simulation's CUDA stream; download/count calls
 *     synchronise it.
 */
#ifndef TECS_GPU_H
#define TECS_GPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Pair finders: include/pair_finders/{naive_all_pairs,binned_all_pairs,naive_gabriel,binned_gabriel,
 *               naive_delaunay}.hpp */
enum tecs_finder {
  TECS_FINDER_NAIVE_ALL_PAIRS = 0,
  TECS_FINDER_BINNED_ALL_PAIRS = 1,
  TECS_FINDER_NAIVE_GABRIEL = 2,
  TECS_FINDER_BINNED_GABRIEL = 3,
  TECS_FINDER_NAIVE_DELAUNAY = 4,   /* naive_delaunay.hpp:31-294; capacity <= 4096, non-symmetric */
  TECS_FINDER_DELAUNAY = 5          /* the same finder for any capacity, from each cell's Delaunay star: in 2-D
                                       the naive finder's multiplicities bit for bit; in 3-D the Delaunay
                                       tetrahedra under its counting rule (its 3-D sphere is centred at
                                       x_i + c, not at the circumcentre c); non-symmetric */
};

/* Integrators: include/integrators/euler.hpp, heun.hpp */
enum tecs_integrator { TECS_EULER = 0, TECS_HEUN = 1 };

/* Built-in pairwise force descriptors (the C layer cannot take user lambdas). */
enum tecs_force {
  TECS_FORCE_NONE = 0,      /* no deltas (pair capture only)                                       */
  TECS_FORCE_SPRING2R = 1,  /* F = k_rep*max(r_rep-d,0) - k_adh*max(d-r_adh,0); covers forces::Spring
                               and forces::PiecewiseLinear (include/forces/predefined.hpp:60-144)   */
  TECS_FORCE_POLARITY = 2   /* spring2r + k_pol*(Polarity_::bending_force + bidirectional alignment)
                               (include/types/polarity.hpp:131-198); dims must be 3                  */
};

/* Simulation description.  Field names and defaults follow Simulation::Settings
 * (include/simulation.hpp:76-98) and BinnedGabriel::Settings
 * (include/pair_finders/binned_gabriel.hpp:20-26). */
typedef struct tecs_sim_desc {
  int dims;                     /* 2 or 3                                                         */
  int finder;                   /* enum tecs_finder                                               */
  int symmetric;                /* 1 = the *Symmetric finder variants (j<i, +d to i, -d to j)     */
  float cutoff;                 /* Settings::cutoff_distance                                      */
  float gabriel_coefficient;    /* default 0.8                                                    */
  float min_bounds[3];          /* default -20                                                    */
  float max_bounds[3];          /* default +20                                                    */
  float bin_size_scale;         /* default 1                                                      */
  int rebuild_every_n;          /* default 0 (rebuild on every full step)                         */
  int integrator;               /* enum tecs_integrator                                           */
  int com_fix;                  /* 0 = com_fixers::NoComFixer, 1 = com_fixers::GlobalComFixer     */
  int force;                    /* enum tecs_force                                                */
  float k_rep, r_rep, k_adh, r_adh, k_pol;
  int has_polarity;             /* second field (Polarity) present                                */
  unsigned capacity;            /* Settings::capacity (>= agent count; COM divides by it)         */
  double division_probability;  /* per cell per step; 0 disables division                         */
  float division_offset;        /* daughter = parent + offset * random unit vector                */
  uint64_t seed;                /* Settings::seed                                                 */
  int device;                   /* CUDA device ordinal                                            */
} tecs_sim_desc;

typedef struct tecs_sim tecs_sim;

/* Fill *desc with the reference defaults (dims 3, binned Gabriel, Heun, no COM). */
int tecs_sim_desc_default(tecs_sim_desc* desc);

/* Simulation(Settings) constructor: allocates the device state for desc->capacity cells.
 * Replaces include/simulation.hpp:133-153. */
int tecs_sim_create(const tecs_sim_desc* desc, tecs_sim** out);

/* Frees every device buffer of the simulation. */
int tecs_sim_destroy(tecs_sim* sim);

/* Initial state from host memory (n <= capacity); resets the finder's
 * rebuild counter as Simulation::set_agent_count does
 * (include/simulation.hpp:295-302).  The division stream stays keyed by the
 * steps taken since creation.  Page-locked buffers are read by the upload
 * kernel directly; other host memory is staged with one copy.  Returns once
 * the buffers may be reused. */
int tecs_sim_upload(tecs_sim* sim, const float* positions, const float* polarity, unsigned n);

/* Same from device memory on the simulation's device (no host copy). */
int tecs_sim_upload_device(tecs_sim* sim, const float* d_positions, const float* d_polarity, unsigned n);

/* Simulation::take_step(dt, force) repeated n_steps times
 * (include/simulation.hpp:548-556 -> integrators/{euler,heun}.hpp::integrate),
 * followed by cell division when enabled.  Asynchronous. */
int tecs_sim_step(tecs_sim* sim, double dt, int n_steps);

/* Wait for the simulation's queued work. */
int tecs_sim_synchronize(tecs_sim* sim);

/* Current agent count (synchronises). */
int tecs_sim_count(tecs_sim* sim, unsigned* n);

/* Copy the state back in cell-id order (synchronises).  The host side of
 * View::sync_host + HDF5_Writer::write (include/io/hdf5_writer.hpp:306-321).
 * positions: capacity*dims floats; polarity: capacity*2 floats or NULL.
 * Page-locked buffers are written by kernels directly (one synchronisation);
 * other host memory receives one staged copy. */
int tecs_sim_download(tecs_sim* sim, float* positions, float* polarity, unsigned* n);

/* Test hook: one full-step force evaluation of the current state with a
 * fresh grid (PairFinder::evaluate_force, e.g. binned_gabriel.hpp:71-362).
 * Writes per-cell deltas in cell-id order (dpos: n*dims, dpol: n*2 or NULL)
 * and, when pairs != NULL, up to pair_capacity directed (self, other) id
 * pairs in unspecified order; *n_pairs receives the total.  Synchronises. */
int tecs_sim_evaluate(tecs_sim* sim, float* dpos, float* dpol, uint32_t* pairs, size_t pair_capacity,
                      size_t* n_pairs);

/* The simulation's CUDA stream (a cudaStream_t). */
void* tecs_sim_stream(tecs_sim* sim);

/* The state in cell-id order into device memory on the simulation's device
 * (positions: capacity*dims floats, polarity: capacity*2 floats or NULL);
 * synchronises.  Replaces View::sync_host's counterpart for device-side
 * user code (include/types/view.hpp:139-148): the drop-in layer's field
 * views read the state from here. */
int tecs_sim_download_device(tecs_sim* sim, float* d_positions, float* d_polarity, unsigned* n);

/* The integrator's old velocities (integrators/base.hpp:59,74), which user
 * pairwise laws that set drag read (binned_gabriel.hpp:225-226, 356-357).
 * keep != 0 allocates them (capacity x 16 bytes, zeroed) and makes every
 * step write them: the step's velocity, d1 - c for Euler (euler.hpp:59),
 * (d1' + d2') * 0.5 for Heun (heun.hpp:87), by cell id.  Keeping them moves
 * the integrator update out of the last force pass into its own kernel;
 * keep == 0 frees them.  Non-symmetric finders only.  Synchronises. */
int tecs_sim_keep_old_velocities(tecs_sim* sim, int keep);
/* The old velocities of the n active cells in cell-id order (out: n*dims
 * floats), *n receiving the count; fails when they are not kept. */
int tecs_sim_old_velocities(tecs_sim* sim, float* out, unsigned* n);
/* Sets the old velocities of cells 0 .. n-1 (v: n*dims floats). */
int tecs_sim_set_old_velocities(tecs_sim* sim, const float* v, unsigned n);

/* Extra fields: a config's fields beyond the position and the polarity
 * (include/simulation_config.hpp:44-192 holds any list of fields), as
 * `components` floats per cell (at most 8; Scalar 1, Polarity 2, Vector
 * dims each), zeroed.  Bit k of double_mask marks component k as a Scalar
 * field's, which the integrators update in double (float += delta * double
 * dt, as the reference's integrators do for a float field).  Every step
 * moves and integrates them with the cell; the built-in laws give them zero
 * deltas, user laws (tecs_sim_set_pair_law) any.  Non-symmetric finders
 * only.  Synchronises. */
int tecs_sim_set_extra_fields(tecs_sim* sim, unsigned components, uint32_t double_mask);
/* One extra field, components [offset, offset + width), of cells 0 .. n-1 in
 * cell-id order (values: n rows of width floats, host or device memory);
 * n <= the active cells. */
int tecs_sim_upload_extra(tecs_sim* sim, unsigned offset, unsigned width, const float* values, unsigned n);
/* The same field of the active cells into out (host or device memory), *n
 * receiving the count. */
int tecs_sim_download_extra(tecs_sim* sim, unsigned offset, unsigned width, float* out, unsigned* n);

/* Device memory for the drop-in layer's views and device variables
 * (include/types/view.hpp:47-266, device_var.hpp:38-134 hold theirs in
 * Kokkos::View device allocations).  tecs_device_copy copies between any two
 * of host and device memory (the direction taken from the addresses) and
 * synchronises. */
int tecs_device_alloc(int device, size_t bytes, void** out);
int tecs_device_free(void* ptr);
int tecs_device_copy(void* dst, const void* src, size_t bytes);

/* Links (include/types/link.hpp): n_links (a, b) cell-id pairs with the
 * constant-pull link law of examples/intercalation.cpp:65-71 -- at every
 * force evaluation cell a gets strength*(x_b - x_a)/|x_b - x_a| and cell b
 * its negative, after the pairwise forces and in link order
 * (integrators/base.hpp:197-234); links with a == b are skipped.  Replaces
 * Settings::link_capacity + get_links() + a LINK_FORCE of that law.  Non-symmetric
 * finders; n_links == 0 removes the links. */
int tecs_sim_set_links(tecs_sim* sim, const uint32_t* links, unsigned n_links, float strength);

/* Change the pairwise force law between steps: take_step(dt, force) with a
 * different force functor (include/simulation.hpp:548-556).  No-op when the
 * law and its constants are unchanged; otherwise waits for queued steps. */
int tecs_sim_set_force(tecs_sim* sim, int force, float k_rep, float r_rep, float k_adh, float r_adh, float k_pol);

/* A user pairwise law (a PAIRWISE_FORCE lambda or functor of the calling
 * program, include/utils/utils.hpp:181-276) in place of the built-in one:
 * for every force evaluation the library calls fn(user, call, stream), and
 * fn launches the pass compiled with the law into the program -- the header
 * include/tecs/pairwise.cuh makes fn for a lambda.  call points to the
 * library's description of the evaluation (its first field is its size in
 * bytes), stream is the simulation's cudaStream_t; fn returns 0 on success.
 * Launches made while a step is captured into a graph replay with it.
 * Non-symmetric all-pairs, Gabriel and Delaunay finders (with the Delaunay
 * finder the library counts each pair's simplices first, and the pass calls
 * the law once per simplex); fn == NULL returns to the built-in law.  Replaces the force argument of take_step
 * (include/simulation.hpp:548-556) for such laws. */
typedef int (*tecs_pair_law_fn)(void* user, const void* call, void* stream);
int tecs_sim_set_pair_law(tecs_sim* sim, tecs_pair_law_fn fn, void* user);

/* Capture each step as a CUDA graph and replay it (default on). */
int tecs_sim_set_graph(tecs_sim* sim, int enable);

/* Bracket every kernel of a step with CUDA events (recorded as event nodes
 * inside the step's graph).  Changing the setting re-captures the graph. */
int tecs_sim_set_profiling(tecs_sim* sim, int enable);

/* Per-kernel durations (ms) of the most recently completed step, in launch
 * order; *count receives the number of kernels (synchronises). */
int tecs_sim_last_step_profile(tecs_sim* sim, float* ms, int capacity, int* count);

/* Name of kernel `index` of that profile (static string), or NULL. */
const char* tecs_sim_profile_name(tecs_sim* sim, int index);

/* Number of kernels one step launches (for launch accounting). */
int tecs_sim_kernels_per_step(tecs_sim* sim, int* kernels);

/* ------------------------------------------------------------------------
 * Engine: many independent simulations advanced together (batched ensemble,
 * served requests).  No counterpart in the reference, which runs one
 * Simulation after another (include/utils/runtime_guard.hpp:26-99 shares the
 * runtime, nothing more).  Each resident simulation is described by the same
 * tecs_sim_desc as a single one (3-D, binned finder, non-symmetric, no COM
 * fix, no division; bin_size_scale >= 1) and evolves exactly as a
 * tecs_sim_step run of it would.  One tecs_engine_step advances every
 * resident simulation by one step of its own integrator in one CUDA graph.
 * ------------------------------------------------------------------------ */
typedef struct tecs_engine_desc {
  unsigned cell_capacity;   /* cells of all resident simulations together */
  unsigned bin_capacity;    /* bins of all resident simulations together  */
  unsigned max_sims;        /* resident simulations at most               */
  int device;
} tecs_engine_desc;

typedef struct tecs_engine tecs_engine;

int tecs_engine_desc_default(tecs_engine_desc* desc);
int tecs_engine_create(const tecs_engine_desc* desc, tecs_engine** out);
int tecs_engine_destroy(tecs_engine* engine);
/* Bins a simulation described by desc occupies in the engine. */
int tecs_engine_bins_needed(const tecs_sim_desc* desc, unsigned* nbins);
/* Free cells and the largest free run of bins (admission by free capacity). */
int tecs_engine_free(tecs_engine* engine, unsigned* free_cells, unsigned* largest_free_bins);
/* Threads per block of the engine's force passes: 64, 96 (the default) or 128.
 * Results do not depend on it; the autotuner (tecs_gb300/batched.py) picks it. */
int tecs_engine_set_pass_threads(tecs_engine* engine, unsigned threads);
/* Admit a simulation with its initial state (host memory); *slot names it. */
int tecs_engine_add(tecs_engine* engine, const tecs_sim_desc* desc, const float* positions, const float* polarity,
                    unsigned n, int* slot);
/* Retire a simulation; its cells and bins are released by the next step. */
int tecs_engine_remove(tecs_engine* engine, int slot);
/* n_steps steps of every resident simulation (asynchronous). */
int tecs_engine_step(tecs_engine* engine, double dt, int n_steps);
int tecs_engine_synchronize(tecs_engine* engine);
/* Resident cells and simulations. */
int tecs_engine_count(tecs_engine* engine, unsigned* cells, unsigned* sims);
/* One simulation's state in cell-id order (synchronises). */
int tecs_engine_download(tecs_engine* engine, int slot, float* positions, float* polarity, unsigned* n);
/* Snapshot into pinned host buffers without stalling the step stream: the
 * cells are unpacked on the device (into staging cells [stage_offset,
 * stage_offset + n)) and copied on a side stream; *event (a cudaEvent_t)
 * completes when the host buffers hold the data. */
int tecs_engine_snapshot_async(tecs_engine* engine, int slot, float* pinned_positions, float* pinned_polarity,
                               unsigned stage_offset, void** event);
int tecs_engine_event_query(void* event, int* ready);
int tecs_engine_event_destroy(void* event);
int tecs_engine_kernels_per_step(tecs_engine* engine, int* kernels);
void* tecs_engine_stream(tecs_engine* engine);

/* ------------------------------------------------------------------------
 * Served stream: a continuous-batching request loop over engines, run by a
 * server thread of this library.  No counterpart in the reference (it runs
 * one Simulation per program).  Requests (a tecs_sim_desc with its state and
 * step count) are submitted from any thread; the server admits each as soon
 * as its lane's engine has free cells and a free run of bins (first come,
 * first served), steps every lane's resident simulations together (each lane
 * on its own stream with at most in_flight step batches queued, never past a
 * resident request's next snapshot or end), writes a snapshot every
 * snapshot_every steps (unpacked on the device, copied to pinned memory on a
 * side stream, written as HDF5 by a writer thread: <dir>/request_<tag>.h5,
 * group t<step>, datasets position and polarity), and retires a request at
 * its step count, keeping its final state for tecs_serve_fetch.
 * ------------------------------------------------------------------------ */
typedef struct tecs_serve_desc {
  int device;
  unsigned cell_capacity;        /* cells of all lanes together                      */
  unsigned bin_capacity;         /* bins of all lanes together                       */
  unsigned max_sims;             /* resident simulations per lane at most            */
  double dt;                     /* the step of every request                        */
  unsigned snapshot_every;       /* 0: no snapshots                                  */
  const char* snapshot_dir;      /* NULL: snapshots are copied but not written       */
  unsigned n_lanes;              /* 1 to 4 size classes                              */
  unsigned lane_max_cells[4];    /* largest request of each lane (last lane: 0, any) */
  float lane_share[4];           /* each lane's share of the capacities              */
  unsigned steps_per_issue;      /* steps per engine call at most (>= 1)             */
  unsigned in_flight;            /* step batches queued per lane at most (>= 1)      */
} tecs_serve_desc;

typedef struct tecs_serve_result {
  uint64_t id;
  uint64_t tag;                  /* the caller's name for the request (submit)       */
  unsigned cells;
  unsigned steps;                /* steps run (the request's, less its start step)   */
  double arrival_s, admitted_s, completed_s;  /* seconds since tecs_serve_create     */
} tecs_serve_result;

typedef struct tecs_serve_stats {
  unsigned long long cell_steps; /* cells x steps of every request so far            */
  unsigned long long engine_steps;
  unsigned long long snapshots_written;
  unsigned long long snapshot_errors;
  unsigned submitted, completed, resident, waiting;
} tecs_serve_stats;

typedef struct tecs_serve tecs_serve;

int tecs_serve_desc_default(tecs_serve_desc* desc);
int tecs_serve_create(const tecs_serve_desc* desc, tecs_serve** out);
/* Queue a request: its state (host memory, copied), its step count and the
 * step it starts from (a resumed request: its snapshots and its end fall on
 * the same steps as in an uninterrupted run).  tag is the caller's name for
 * it: its snapshots go to <snapshot_dir>/request_<tag, 5 digits>.h5 (a new
 * file).  *id receives the server's name for it. */
int tecs_serve_submit(tecs_serve* server, const tecs_sim_desc* desc, const float* positions, const float* polarity,
                      unsigned n, unsigned steps, unsigned start_step, uint64_t tag, uint64_t* id);
/* Results completed since the last call, up to capacity; *n receives the count. */
int tecs_serve_poll(tecs_serve* server, tecs_serve_result* results, unsigned capacity, unsigned* n);
/* A completed request's final state in cell-id order; fails for an unknown or
 * unfinished request.  The state is released after the fetch. */
int tecs_serve_fetch(tecs_serve* server, uint64_t id, float* positions, float* polarity, unsigned* n);
/* Waits until every submitted request has completed and every snapshot is
 * written, or timeout_s passes (then fails). */
int tecs_serve_drain(tecs_serve* server, double timeout_s);
int tecs_serve_stats_get(tecs_serve* server, tecs_serve_stats* stats);
/* Stops the server thread (resident requests are dropped) and frees everything. */
int tecs_serve_destroy(tecs_serve* server);

/* ------------------------------------------------------------------------
 * Standalone bin grid: acceleration::Grid (include/utils/grid.hpp:29-638),
 * the grid user forces query for the nearest point or a random neighbour
 * (examples/tribolium/main.cpp:84-95, intercalation_w_gradient.cpp:73-91).
 * Bins of bin_size over [min_bounds, max_bounds) (ceil((max-min)/bin_size)
 * per axis, grid.hpp:201-206); a point's bin is clamp(int((p-min)/bin_size))
 * (grid.hpp:222-230).  Points are sorted by (bin, index) on every rebuild.
 * ------------------------------------------------------------------------ */
typedef struct tecs_grid tecs_grid;

enum tecs_grid_query_kind {
  TECS_GRID_NEAREST = 0,          /* get_nearest_point_index(point, radius_bins), grid.hpp:413-441            */
  TECS_GRID_RANDOM_IN_BINS = 1,   /* get_random_point_index_in_neighbourhood_bins(point, radius_bins, rng),
                                     grid.hpp:453-492                                                        */
  TECS_GRID_RANDOM_IN_RADIUS = 2  /* get_random_point_index_in_neighbourhood(point, radius, rng[, filter]),
                                     grid.hpp:505-637                                                        */
};

/* A grid for up to `capacity` points of `dims` (2 or 3) coordinates. */
int tecs_grid_create(int dims, const float* min_bounds, const float* max_bounds, float bin_size, unsigned capacity,
                     int device, tecs_grid** out);
int tecs_grid_destroy(tecs_grid* grid);
/* Grid::rebuild (grid.hpp:389-401) over n points float[n][dims] in host
 * memory; synchronises. */
int tecs_grid_rebuild(tecs_grid* grid, const float* points, unsigned n);
/* The same from device memory on the grid's device. */
int tecs_grid_rebuild_device(tecs_grid* grid, const float* d_points, unsigned n);
/* m queries (host arrays): out[q] = the point index the reference's query
 * returns at queries[q], or -1.  The random kinds take draws[q] for the
 * reference's rng.rand(0, total) / rng.urand(total): the target is
 * draws[q] mod total.  eligible (host, one byte per point, or NULL) is the
 * filter of the radius query: points with eligible[index] == 0 are skipped.
 * Synchronises. */
int tecs_grid_query(tecs_grid* grid, int kind, const float* queries, unsigned m, int radius_bins, float radius,
                    const uint32_t* draws, const uint8_t* eligible, int32_t* out);
/* Device arrays of the last rebuild, for device code that queries the grid
 * itself (tecs/device/grid_query.cuh): positions sorted by (bin, index)
 * (float4, w = bin key), the index of each sorted slot, and the nbins + 1
 * bin offsets. */
int tecs_grid_device_view(const tecs_grid* grid, const void** sorted_positions, const unsigned** sorted_index,
                          const unsigned** bin_offsets);

/* Limits of tecs_force_pass_noalloc (its scratch is a fixed static device array). */
#define TECS_NOALLOC_MAX_CELLS 65536u
#define TECS_NOALLOC_MAX_BINS 262144u

/* No counterpart in the reference: an allocation-free form of the one-pass
 * force evaluation of tecs_sim_evaluate, for callers that may not allocate
 * device memory (a host runtime that owns the GPU memory budget, a serving
 * loop that must not stall on or fragment the allocator).  Reads positions
 * (device, float[n][dims]), writes per-cell deltas (device, float[n][dims],
 * input order) for a binned, non-symmetric finder with the spring law or no
 * force, queued on `stream` (a cudaStream_t, 0 = legacy default).  Allocates
 * nothing: its scratch is a static device array of about 6 MB that every GPU
 * loading the library keeps until exit.  Rejects more than
 * TECS_NOALLOC_MAX_CELLS cells or TECS_NOALLOC_MAX_BINS bins.  Runs on
 * desc->device, which it makes current like the other entry points; the
 * buffers and the stream must belong to that device.  The first call on a
 * device looks up the array's device address (once per device, kept for the
 * life of the process: resetting the device in between is not supported), so
 * make that first call before any stream capture.  All calls on a device share
 * the array: calls whose GPU work overlaps race and must be serialised. */
int tecs_force_pass_noalloc(const tecs_sim_desc* desc, const float* d_positions, unsigned n, float* d_deltas,
                            void* stream);

/* Message of the last failing call on this thread. */
const char* tecs_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* TECS_GPU_H */

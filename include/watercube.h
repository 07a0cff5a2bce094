/*
 * watercube.h — C ABI of the GB300 SPH water solver.
 *
 * This is the drop-in boundary for WaterCube's simulation path. The reference exposes it as the
 * C++ class core::Fluid (src/core/Fluid.h:32-141) driving the GLSL compute shaders through
 * core::Sort (src/core/Sort.h:20-39) and util::runProg (src/core/util.cpp:32-36). Every entry
 * point below names the reference member it replaces. All entry points are plain C: POD structs,
 * plain pointers and sizes, a status code, and a thread-local error message.
 *
 * Buffers (all device memory is owned by the library; see wc_device_buffers):
 *   state buffer   = the reference's particle_buffer1_ (Fluid.h:135): particles after update(),
 *                    stored in the order of the last sort, exactly as the reference leaves them.
 *   sorted buffer  = particle_buffer2_ (Fluid.h:136): Sort::run's output, density written in place.
 *   cell tables    = Sort's count_buffer_/offset_buffer_ (Sort.h:70), sized by the cell count.
 * The library stores particles as SoA float4 pairs (position+density, velocity+pressure), which
 * holds the same 32 bytes per particle as the reference's AoS `struct Particle` (util.h:29-35).
 * wc_particle is that AoS struct, used for host copies.
 *
 * Threading: a wc_fluid is not thread-safe. All work is enqueued on the handle's own CUDA stream;
 * wc_fluid_update returns without waiting, and every copy-to-host call synchronises that stream.
 */
#ifndef WATERCUBE_H
#define WATERCUBE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define WC_API __attribute__((visibility("default")))
#else
#define WC_API
#endif

#define WC_API_VERSION 1

/* Status codes. The reference has none (it asserts, src/core/Fluid.cpp:222-223). */
typedef enum wc_status {
    WC_OK = 0,
    WC_ERR_INVALID_ARG = 1, /* bad parameter, size or pointer */
    WC_ERR_OOM = 2,         /* device or pinned host allocation failed */
    WC_ERR_CUDA = 3,        /* a CUDA runtime call failed (no device, launch error, ...) */
    WC_ERR_TIMEOUT = 4,     /* a bounded device-side wait gave up (prefix-scan look-back) */
    WC_ERR_NUMERIC = 5,     /* a non-finite particle position was binned */
    WC_ERR_STATE = 6,       /* call out of order (e.g. update before setup) */
    WC_ERR_UNSUPPORTED = 7  /* feature not compiled in */
} wc_status;

/* Equation of state. */
enum {
    /* p = p0 + k((rho/rho0)^3 - 1): Desbrun & Cani form, the one the reference runs
       (assets/fluid/density.comp:130-133). */
    WC_EOS_DESBRUN_CUBIC = 0,
    /* p = p0 + k(rho - rho0): the reference's commented-out Harada form (density.comp:129). */
    WC_EOS_LINEAR = 1
};

/* Behaviour switches. The reference runs with the first four on. */
enum {
    WC_FLAG_WALL_DENSITY = 1u << 0, /* pseudo wall density, x4 (density.comp:57-79, incl. its z branch testing y) */
    WC_FLAG_WALL_FORCE = 1u << 1,   /* spiky wall push, x0.01 (update.comp:71-100) */
    WC_FLAG_SPEED_CLAMP = 1u << 2,  /* per-component velocity clamp to +-max_speed (update.comp:5,199) */
    WC_FLAG_MOUSE_FORCE = 1u << 3,  /* repulsion from the mouse ray (update.comp:116-132) */
    WC_FLAG_TRACK_IDS = 1u << 4,    /* carry each particle's original index through every sort */
    WC_FLAG_NEIGHBOR_COUNTS = 1u << 5, /* write per-particle neighbour counts in the density pass */
    /* Boundary handling by wall weight functions (Harada et al. 2007), in closed form for a
       continuous planar wall of rest density at each face of the box: a particle at distance
       d < h from a wall gains rho0 * 315/256 * P(1 - d/h) of density, with
       P(x) = x^5 (16/5 - 16x/3 + 24x^2/7 - x^3 + x^4/9) (half the kernel's mass at d = 0), which
       enters the equation of state; and, when its pressure is positive, the mirrored pressure
       push (p rho0 / rho) * (30/h) * (x^4/4 - x^5/5) away from the wall (the surface integral
       of the Spiky kernel over the wall plane). No counterpart in the reference: the
       replacement for its pseudo wall density and force that its report names as the next
       physics fix. */
    WC_FLAG_WALL_WEIGHTS = 1u << 6,
    /* Run both neighbour passes (density, force) as one 32-lane team per non-empty cell
       (WC_PASSES_TEAM) instead of one lane per target (the default, WC_PASSES_LANE); the same
       neighbour sets, the sums differ only in the order of their additions. */
    WC_FLAG_CELL_TEAMS = 1u << 7
};

/* The reference's four active behaviours. */
#define WC_FLAGS_REFERENCE (WC_FLAG_WALL_DENSITY | WC_FLAG_WALL_FORCE | WC_FLAG_SPEED_CLAMP | WC_FLAG_MOUSE_FORCE)

/*
 * Simulation parameters: the reference's fluent setters (Fluid.h:37-48) and the constants
 * Fluid::setup derives (Fluid.cpp:203-216). Fill with a preset, change fields, then
 * wc_params_finalize derives the zero fields.
 */
typedef struct wc_params {
    uint32_t num_particles; /* Fluid::numParticles */
    uint32_t grid_res;      /* Fluid::gridRes: cells per axis. 0 -> floor(size / kernel_radius) */
    float size;             /* Fluid::size: the domain is [0,size]^3 */
    float particle_radius;  /* Fluid::particleRadius */
    float kernel_radius;    /* h. 0 -> 4 * particle_radius (Fluid.cpp:209) */
    float particle_mass;    /* m. 0 -> 8 * particle_radius (Fluid.cpp:210) */
    float rest_density;     /* Fluid::restDensity */
    float rest_pressure;    /* Fluid::restPressure */
    float stiffness;        /* Fluid::stiffness */
    float viscosity;        /* Fluid::viscosityCoefficient */
    float gravity[3];       /* gravity_direction_ * gravity_strength_ (Fluid.cpp:310) */
    float time_scale;       /* wc_fluid_update(time) integrates dt = float(time) * time_scale (Fluid.cpp:308) */
    uint32_t eos;           /* WC_EOS_* */
    uint32_t flags;         /* WC_FLAG_* */
    float max_speed;        /* speed clamp, 50 in the reference (update.comp:5) */
    float wall_damping;     /* velocity factor on wall contact: v *= -wall_damping (update.comp:202) */
    float wall_border;      /* wall clamp distance (update.comp:203) */
    float mouse_origin[3];  /* mouse ray, in the fluid's frame (Fluid::getRelativeMouseRay) */
    float mouse_dir[3];
    /* Derived by wc_params_finalize when zero: */
    float bin_size;    /* size / grid_res (Fluid.cpp:208) */
    float poly6_const; /* 315 / (64 pi h^9), computed in double, cast to float (Fluid.cpp:214) */
    float spiky_const; /* -45 / (pi h^6) (Fluid.cpp:215) */
    float visc_const;  /* 45 / (pi h^6) (Fluid.cpp:216) */
    uint32_t reserved[4];
} wc_params;

/* AoS particle, bit-compatible with the reference's std430 `struct Particle` (util.h:29-35). */
typedef struct wc_particle {
    float position[3];
    float density;
    float velocity[3];
    float pressure;
} wc_particle;

/* Which particle buffer a host copy reads or writes. */
enum {
    WC_BUFFER_STATE = 1, /* particle_buffer1_: the state update() leaves behind */
    WC_BUFFER_SORTED = 2 /* particle_buffer2_: the sort's output (density/pressure after the density pass) */
};

/* Integer buffers a host copy can read (util::getUints, src/core/util.cpp:62-72). */
enum {
    WC_UINTS_CELL_KEYS = 1,      /* per input particle: its cell key (count.comp:31-33) */
    WC_UINTS_PERMUTATION = 2,    /* per sorted slot: input index it came from (sort.comp:44) */
    WC_UINTS_CELL_COUNTS = 3,    /* per cell: particle count (Sort::getCountBuffer) */
    WC_UINTS_CELL_OFFSETS = 4,   /* per cell: exclusive prefix of counts (Sort::getOffsetBuffer) */
    WC_UINTS_NEIGHBOR_COUNTS = 5,/* per sorted particle: neighbours j != i with |r| < h (needs WC_FLAG_NEIGHBOR_COUNTS) */
    WC_UINTS_PARTICLE_IDS = 6    /* per state-buffer particle: original index (needs WC_FLAG_TRACK_IDS) */
};

/* Raw device pointers, borrowed: valid until the next wc_fluid_* call that runs a step, or destroy. */
typedef struct wc_device_buffers {
    void* state_pos_density;    /* float4[n]: x, y, z, density     (state buffer) */
    void* state_vel_pressure;   /* float4[n]: vx, vy, vz, pressure (state buffer) */
    void* sorted_pos_density;   /* float4[n]  (sorted buffer) */
    void* sorted_vel_pressure;  /* float4[n]  (sorted buffer) */
    void* cell_keys;            /* uint32[n] */
    void* permutation;          /* uint32[n] */
    void* cell_start;           /* uint32[num_cells + 1]: cell c holds sorted slots [start[c], start[c+1]) */
    void* neighbor_counts;      /* uint32[n] or NULL */
    void* particle_ids;         /* uint32[n] or NULL */
    void* stream;               /* cudaStream_t the handle enqueues on */
    uint32_t num_particles;
    uint32_t num_cells;
} wc_device_buffers;

typedef struct wc_fluid wc_fluid;

/* ---- parameters ---------------------------------------------------------------------------- */

/* The reference's constructor defaults (src/core/Fluid.cpp:9-27): 80,000 particles, gridRes 21,
   r = 0.01, rho0 = 500, mu = 200, k = 100, p0 = 0, g = 900 down, time scale 0.012, cubic EOS,
   WC_FLAGS_REFERENCE, a mouse ray that misses the box. */
WC_API void wc_params_reference_defaults(wc_params* p);

/* Dam-break preset: unit box, h = 0.0457 * (16384/n)^(1/3), lattice spacing h/2,
   m = 1000 (h/2)^3, rho0 = 1000, k = 3, mu = 3.5, g = (0,-9.81,0), linear EOS, restitution 0.5,
   no reference-only extras, grid_res = floor(1/h). n = 16384 and n = 1048576 are the two sizes
   this solver is benchmarked at. */
WC_API void wc_params_dam_break(wc_params* p, uint32_t num_particles);

/* Fill derived fields and validate. WC_ERR_INVALID_ARG when the grid cannot hold the kernel
   (bin_size < kernel_radius) or a value is out of range. */
WC_API wc_status wc_params_finalize(wc_params* p);

/* Largest float x with sqrtf(x) < h: |r| < h  <=>  dot(r,r) <= this (exact for IEEE sqrt). */
WC_API float wc_cull_threshold(float kernel_radius);

/* ---- initial states (host only) ---------------------------------------------------------- */

/* The reference's dam-break lattice (Fluid::generateInitialParticles, Fluid.cpp:104-134):
   ceil(cbrt(n)) per side, spacing 1.75 r, jitter in [-0.25, 0.25) * spacing per component.
   MSVC rand() is replaced by splitmix64(seed). */
WC_API wc_status wc_generate_reference_lattice(const wc_params* p, uint64_t seed, wc_particle* out, uint32_t n);

/* The dam-break preset's block: spacing s = h/2, nx = nz = floor(cbrt(n/2)), ny = ceil(n/(nx nz)),
   site (i,j,k) at ((i+.5)s, (j+.5)s, (k+.5)s) filled x fastest, then z, then y; first n sites;
   each component jittered by (2u-1) * 0.01 h with u = top 24 bits of splitmix64(seed) * 2^-24,
   three draws per particle in x, y, z order. */
WC_API wc_status wc_generate_dam_break(const wc_params* p, uint64_t seed, wc_particle* out, uint32_t n);

/* ---- the fluid (core::Fluid) ------------------------------------------------------------- */

/* Fluid::create + the fluent setters: copies params (finalizing them) and allocates every device
   buffer. Fails with WC_ERR_CUDA when no CUDA device is present. */
WC_API wc_status wc_fluid_create(const wc_params* p, wc_fluid** out);

/* Fluid::setup's buffer upload (Fluid.cpp:139-166): copy n == num_particles initial particles
   into the state buffer. Must be called once before the first step; may be called again to reset. */
WC_API wc_status wc_fluid_setup(wc_fluid* f, const wc_particle* initial, uint32_t n);

/* Fluid::update(double time) (Fluid.cpp:342-354): sort, density, forces+integration with
   dt = float(time) * time_scale. Asynchronous on the handle's stream (CUDA-graph launched). */
WC_API wc_status wc_fluid_update(wc_fluid* f, double time);

/* nsteps updates with dt given directly (time_scale not applied). */
WC_API wc_status wc_fluid_step(wc_fluid* f, float dt, uint32_t nsteps);

/* The three stages of one update, for inspection: Sort::run (Sort.cpp:254-267),
   Fluid::runDensityProg (Fluid.cpp:268-289), Fluid::runUpdateProg (Fluid.cpp:294-321). */
WC_API wc_status wc_fluid_sort(wc_fluid* f);
WC_API wc_status wc_fluid_density(wc_fluid* f);
WC_API wc_status wc_fluid_integrate(wc_fluid* f, float dt);

/* Fluid::setMouseRay (Fluid.h:52) in the fluid's own frame. */
WC_API wc_status wc_fluid_set_mouse_ray(wc_fluid* f, const float origin[3], const float dir[3]);
/* gravity_direction_ * gravity_strength_ (Fluid::updateGravity / gravityStrength). */
WC_API wc_status wc_fluid_set_gravity(wc_fluid* f, const float gravity[3]);

/* util::getParticles (util.cpp:42-60): synchronise and copy n particles of a buffer to host. */
WC_API wc_status wc_fluid_get_particles(wc_fluid* f, int buffer, wc_particle* out, uint32_t n);
/* util::setParticles (util.cpp:74-78): overwrite a buffer from host. With WC_FLAG_TRACK_IDS,
   writing the state buffer restarts the particle ids at the uploaded order (id = index). */
WC_API wc_status wc_fluid_set_particles(wc_fluid* f, int buffer, const wc_particle* in, uint32_t n);

/* One update with host buffers, the three calls a host-side caller makes per frame in one:
   wc_fluid_set_particles(WC_BUFFER_STATE, in) (skipped when in is null), wc_fluid_update(time)
   and wc_fluid_get_particles(WC_BUFFER_STATE, out) (skipped when out is null), with the same
   results bit for bit. The readback overlaps the step: the force pass writes the host records
   of the particles it stores and flags each eighth of the slots in mapped host memory once it
   is complete, and the calling thread copies that part out while the pass computes the rest
   (lane passes; with WC_FLAG_CELL_TEAMS the copy follows the step). Pinned host memory
   (cudaMallocHost, wc_alloc_host) lets the copies run alongside; pageable memory gives the same
   results without the overlap. Returns after the copy to out has landed (or, with out null,
   like wc_fluid_update). */
WC_API wc_status wc_fluid_update_host(wc_fluid* f, double time, const wc_particle* in, wc_particle* out, uint32_t n);
/* util::getUints (util.cpp:62-72): synchronise and copy an integer buffer (WC_UINTS_*). n must
   equal its length: num_particles, or num_cells for the two cell tables. */
WC_API wc_status wc_fluid_get_uints(wc_fluid* f, int which, uint32_t* out, size_t n);

WC_API wc_status wc_fluid_get_params(const wc_fluid* f, wc_params* out);
WC_API wc_status wc_fluid_get_device_buffers(wc_fluid* f, wc_device_buffers* out);

/* Wait for the handle's stream and report any device-side error flag raised since the last call
   (WC_ERR_NUMERIC, WC_ERR_TIMEOUT). */
WC_API wc_status wc_fluid_synchronize(wc_fluid* f);

/* As wc_batch_set_recording / wc_batch_get_accelerations, for one fluid. */
WC_API wc_status wc_fluid_set_recording(wc_fluid* f, int on);
WC_API wc_status wc_fluid_get_accelerations(wc_fluid* f, float* out /* n x 4 */, uint32_t n);

/* Steps taken since setup. */
WC_API uint64_t wc_fluid_step_count(const wc_fluid* f);

WC_API void wc_fluid_destroy(wc_fluid* f);

/* ---- timing (CUDA events on the handle's stream) ---------------------------------------- */

/* Number of kernels one step launches, and their names (index 0 .. count-1). */
WC_API uint32_t wc_step_kernel_count(void);
WC_API const char* wc_step_kernel_name(uint32_t index);

/*
 * Run nsteps steps of dt, each preceded (outside its timed span) by an L2 flush when flush_l2 is
 * non-zero. step_ms[s] receives the device time of step s (graph launch, CUDA events).
 * kernel_ms, when not NULL, receives nsteps * wc_step_kernel_count() per-kernel times from a
 * further nsteps separately launched steps with an event between kernels (after the graph
 * steps when step_ms is given; alone when step_ms is NULL). At least one of the two is given.
 */
WC_API wc_status wc_fluid_time_steps(wc_fluid* f, float dt, uint32_t nsteps, int flush_l2, float* step_ms,
                                     float* kernel_ms);

/* ---- batches of independent scenes ---------------------------------------------------- */
/*
 * No counterpart in the reference (which simulates one scene). Hundreds of independent scenes
 * with their own particle counts, kernel radius, grid and constants advance together: one
 * global cell sort and one launch per stage for all scenes, replayed as one CUDA graph. Scene s
 * keeps its particles in slots [offset[s], offset[s+1]) of the concatenated buffers.
 */
typedef struct wc_batch wc_batch;

/* A scene of the batched workload: a fluid block of num_particles on a cubic lattice of spacing
   s = (V_block / num_particles)^(1/3), h = 2 s, m = rest_density s^3, velocities N(0, sigma). */
typedef struct wc_scene_spec {
    uint32_t num_particles;
    float block_min[3];
    float block_max[3];
    float stiffness;
    float velocity_sigma;
    uint64_t seed;
} wc_scene_spec;

/* The 512-scene workload's scene draw: counts log-uniform in [n_min, n_max], block sides
   uniform in [0.2, 0.7] standing on the floor at a uniform x/z offset, stiffness uniform in
   [2, 6], velocity sigma 0.5; all from splitmix64(seed). */
WC_API wc_status wc_generate_batch_specs(uint64_t seed, uint32_t num_scenes, uint32_t n_min, uint32_t n_max,
                                         wc_scene_spec* out);
/* Finalized parameters of a scene: the dam-break preset's constants with the spec's h, m, k. */
WC_API wc_status wc_scene_params(const wc_scene_spec* spec, wc_params* out);
/* The scene's initial particles (num_particles entries). */
WC_API wc_status wc_generate_scene(const wc_scene_spec* spec, const wc_params* p, wc_particle* out);

WC_API wc_status wc_batch_create(const wc_params* scenes, uint32_t num_scenes, wc_batch** out);
/* Upload all scenes' initial particles, concatenated in scene order (total entries). */
WC_API wc_status wc_batch_setup(wc_batch* b, const wc_particle* initial, uint64_t total);
WC_API wc_status wc_batch_step(wc_batch* b, float dt, uint32_t nsteps);
WC_API wc_status wc_batch_get_particles(wc_batch* b, wc_particle* out, uint64_t total);
WC_API wc_status wc_batch_set_particles(wc_batch* b, const wc_particle* in, uint64_t total);
/* One step with host buffers, as wc_fluid_update_host: wc_batch_set_particles(in) (skipped when
   in is null), wc_batch_step(dt, 1) and wc_batch_get_particles(out) (skipped when out is null),
   the same results bit for bit, the readback overlapping the force pass (lane passes). */
WC_API wc_status wc_batch_step_host(wc_batch* b, float dt, const wc_particle* in, wc_particle* out, uint64_t total);
/* offsets[num_scenes + 1]: scene s owns slots [offsets[s], offsets[s+1]). */
WC_API wc_status wc_batch_scene_offsets(const wc_batch* b, uint64_t* offsets);
WC_API uint32_t wc_batch_num_scenes(const wc_batch* b);
WC_API uint64_t wc_batch_num_particles(const wc_batch* b);
/* Per-scene FP64 reductions on the device: out[6 s + 0..5] = mass, momentum x/y/z, kinetic
   energy, potential energy (-m g.x summed). */
WC_API wc_status wc_batch_diagnostics(wc_batch* b, double* out);
WC_API wc_status wc_batch_time_steps(wc_batch* b, float dt, uint32_t nsteps, int flush_l2, float* step_ms);
WC_API wc_status wc_batch_device_buffers(wc_batch* b, wc_device_buffers* out);
/* Training-data recording: when on, every step also stores each particle's SPH acceleration
   (forces / density, before the speed clamp and wall collision), in the state buffer's order. */
WC_API wc_status wc_batch_set_recording(wc_batch* b, int on);
WC_API wc_status wc_batch_get_accelerations(wc_batch* b, float* out /* total x 4 */, uint64_t total);
/* Original index (global slot at setup) of each state-buffer particle. */
WC_API wc_status wc_batch_get_ids(wc_batch* b, uint32_t* out, uint64_t total);
WC_API void wc_batch_destroy(wc_batch* b);

/* Launch geometry the autotuner picks: resident blocks per SM of the two neighbour passes and
   of the per-particle kernels, and the cell edge as a multiple of each scene's h. */
/* Neighbour pass variants (threads per cell): one 32-lane team per non-empty cell, its targets
   split into slices, or one lane per target. Same neighbour sets; sums differ in addition order
   only. */
#define WC_PASSES_TEAM 0
#define WC_PASSES_LANE 1

typedef struct wc_tuning {
    uint32_t density_blocks_per_sm;
    uint32_t force_blocks_per_sm;
    uint32_t stream_blocks_per_sm;
    float cell_factor;
    float step_ms; /* best measured step time */
    uint32_t trials;
    uint32_t pass_variant; /* WC_PASSES_TEAM or WC_PASSES_LANE */
} wc_tuning;

/* Time graph replays of candidate geometries (the state is saved before and restored after,
   so the simulation does not advance) and keep the fastest; results are cached per
   (particle count, particles per cell) for the process, and in the file named by
   $WC_TUNE_CACHE when set. */
WC_API wc_status wc_batch_tune(wc_batch* b, float dt, wc_tuning* out);
WC_API wc_status wc_batch_set_tuning(wc_batch* b, const wc_tuning* t);
WC_API wc_status wc_batch_get_tuning(const wc_batch* b, wc_tuning* out);

/* ---- snapshots ---------------------------------------------------------------------------- */
/*
 * No counterpart in the reference (Fluid::reset is a no-op, Fluid.h:57). A snapshot holds a
 * fluid's state buffer (SoA float4 position+density and velocity+pressure, in the order of the
 * last sort), its particle ids when tracked, the step count and the parameters (with the
 * gravity and mouse ray in effect), followed by an FNV-1a 64 checksum of all preceding bytes.
 * A fluid loaded from a snapshot continues bit for bit.
 */
typedef struct wc_snapshot_header {
    char magic[8];          /* "WCSNAP\0\1" */
    uint32_t version;       /* 1 */
    uint32_t header_bytes;  /* sizeof(wc_snapshot_header) */
    uint64_t num_particles;
    uint64_t step;          /* wc_fluid_step_count when saved */
    uint64_t seed;          /* the caller's seed of the initial state, informational */
    uint32_t has_ids;       /* 1: uint32 ids[n] follow the two float4 arrays */
    uint32_t reserved;
    wc_params params;
} wc_snapshot_header;

WC_API wc_status wc_fluid_save_snapshot(wc_fluid* f, const char* path, uint64_t seed);
/* Reads and verifies a snapshot (magic, version, sizes, checksum); fills the header. */
WC_API wc_status wc_snapshot_read_header(const char* path, wc_snapshot_header* out);
/* Load into a fluid created with the same parameters (gravity and mouse ray excepted: they are
   taken from the snapshot). */
WC_API wc_status wc_fluid_load_snapshot(wc_fluid* f, const char* path);
WC_API wc_status wc_fluid_create_from_snapshot(const char* path, wc_fluid** out);

/* ---- surface extraction ------------------------------------------------------------------ */
/*
 * No counterpart in the reference (it draws particles as points; surface reconstruction is its
 * report's stated future work). A colour field phi(v) = sum_j (m / rho0) W_poly6(|v - x_j|, r)
 * is evaluated on grid_res^3 vertices spanning [0, size]^3 (about 1 inside the fluid), and
 * marching cubes extracts the iso-surface phi = iso as a triangle soup (9 floats per triangle,
 * counter-clockwise seen from outside the fluid). Vertices shared by neighbouring cubes are
 * bit-identical, so the mesh is watertight.
 */
typedef struct wc_surface wc_surface;
typedef struct wc_surface_params {
    uint32_t grid_res; /* vertices per axis, 2..1024 */
    float iso;         /* iso-level of the colour field (0.5: half the rest density) */
    float radius;      /* field kernel radius; 0 -> the fluid's h (at most the cell edge) */
    uint32_t reserved;
} wc_surface_params;

WC_API wc_status wc_surface_create(const wc_surface_params* p, wc_surface** out);
WC_API void wc_surface_destroy(wc_surface* s);
/* Sort the fluid's current state, evaluate the field and build the mesh on the device. */
WC_API wc_status wc_surface_extract(wc_surface* s, wc_fluid* f, uint64_t* num_triangles);
WC_API wc_status wc_surface_get_triangles(wc_surface* s, float* out /* 9 x num_triangles */, uint64_t num_triangles);
WC_API wc_status wc_surface_get_field(wc_surface* s, float* out /* grid_res^3, x fastest */, uint64_t count);
/* CUDA-event times of the last extraction: field kernel, and classify + scan + emit. */
WC_API wc_status wc_surface_timings(const wc_surface* s, float* ms_field, float* ms_mesh);
/* The generated marching-cubes case table: counts[256], tris[256][36] (edge ids, -1 unused). */
WC_API wc_status wc_surface_case_table(uint8_t* counts, int8_t* tris);

/* ---- learned surrogate: network operations ---------------------------------------------- */
/*
 * No counterpart in the reference. Building blocks of the message-passing surrogate; all
 * pointers are device memory; work is enqueued on `stream`; device-side failures (a bounded
 * tensor-core wait that ran out) are OR-ed into *d_err (WC_DEVERR_* bits) when d_err is set.
 */
#define WC_DEVERR_MMA_TIMEOUT 4u

/* C = A . B (+ bias) (+ add1[add1_idx[row]] + add2[add2_idx[row]]) (ReLU) on the tensor cores
   (BF16 operands, FP32 accumulation), 128 x 128 output tiles. */
typedef struct wc_gemm_desc {
    uint32_t m, n, k;      /* k a multiple of 8, unless A is transposed and B row-major */
    uint32_t k_chunk;      /* K range per split (multiple of 64; >= k for no split) */
    const void* a;         /* bf16 */
    const void* a2;        /* bf16 second source for A columns >= k_split, or NULL */
    const uint32_t* a_rows;/* A row gather, or NULL */
    uint32_t lda, lda2, k_split;
    int a_transposed;      /* 0: A row-major [m x k]; 1: A[i][kk] = a[kk * lda + i] */
    const void* b;         /* bf16 */
    uint32_t ldb;
    int b_rowmajor;        /* 0: b holds B^T [n x k] row-major; 1: b holds B [k x n] row-major */
    const float* bias;     /* [n] or NULL */
    const void* add1;      /* bf16 rows added in the epilogue, or NULL */
    const uint32_t* add1_idx;
    const void* add2;
    const uint32_t* add2_idx;
    uint32_t ld_add;
    int relu;
    float* c_f32;          /* fp32 output (split s at c_f32 + s * split_stride), or NULL */
    void* c_bf16;          /* bf16 output, or NULL */
    uint32_t ldc;
    size_t split_stride;
    int accumulate;        /* non-zero: c_f32 += result */
    /* LayerNorm epilogue when ln_gamma is set (n = 128, plain row-major A and B^T, BF16 output
       only, no ReLU, gathers or accumulation): c_bf16 = LN(A . B (+ bias)) * ln_gamma + ln_beta
       (+ ln_resid, BF16 rows of 128), the row's mean and variance over its 128 columns in FP32,
       epsilon 1e-5 */
    const float* ln_gamma;
    const float* ln_beta;
    const void* ln_resid;  /* bf16, or NULL */
} wc_gemm_desc;

WC_API wc_status wc_nn_gemm(const wc_gemm_desc* g, uint32_t* d_err, void* stream);

/* ---- learned surrogate: network, training and judged rollout ---------------------------- */
/*
 * No counterpart in the reference. A message-passing network over the radius-h graph of a
 * fluid (latent width 128, `layers` message-passing steps) predicts each particle's SPH
 * acceleration from its last five velocities (the current one and four differences / dt),
 * its wall distances and the scene's stiffness.
 * Inputs and outputs are in the fluid's state-buffer order; the network works in the sorted
 * order internally.
 */
typedef struct wc_surrogate wc_surrogate;

typedef struct wc_surrogate_config {
    uint32_t layers;      /* message-passing steps (default 8) */
    uint64_t seed;        /* weight initialisation */
    float velocity_scale; /* velocities are divided by this in the features (default 1) */
    float accel_scale;    /* network outputs are multiplied by this (default 10) */
} wc_surrogate_config;

WC_API void wc_surrogate_config_default(wc_surrogate_config* c);
WC_API wc_status wc_surrogate_create(const wc_surrogate_config* c, wc_surrogate** out);
WC_API void wc_surrogate_destroy(wc_surrogate* s);
/* FP32 master weights, all layers in one buffer (Adam runs over it in one launch). */
WC_API uint64_t wc_surrogate_num_params(const wc_surrogate* s);
WC_API wc_status wc_surrogate_get_params(wc_surrogate* s, float* host, uint64_t n);
WC_API wc_status wc_surrogate_set_params(wc_surrogate* s, const float* host, uint64_t n);
/* Gradients accumulated since the last wc_surrogate_adam / wc_surrogate_zero_grads. */
WC_API wc_status wc_surrogate_get_grads(wc_surrogate* s, float* host, uint64_t n);
WC_API wc_status wc_surrogate_zero_grads(wc_surrogate* s);
/* Load one training sample: the fluid's current particles (positions and velocities, set
   with wc_fluid_set_particles), the velocity history hist[5][n][4] (hist[0] = current
   velocity, hist[k] = k steps ago, dt apart), optionally the target accelerations
   target[n][4], and optionally the last SPH acceleration stale[n][4] computed stale_age >= 1
   steps ago (NULL or 0: none; the network then sees zeros there). A sample with a stale
   acceleration is residual: the network's output stands for the change since then (its loss
   target is target - stale) and wc_surrogate_predictions returns stale + output. Sorts the
   fluid and builds the graph and features. */
WC_API wc_status wc_surrogate_sample(wc_surrogate* s, wc_fluid* f, float dt, const float* hist, const float* target,
                                     const float* stale, uint32_t stale_age);
/* Forward pass on the loaded sample; with do_backward, the gradients of the mean squared error
   (per component, outputs scaled by 1 / accel_scale) are added to the accumulated ones. *loss
   (may be NULL) receives that error. */
WC_API wc_status wc_surrogate_forward_backward(wc_surrogate* s, int do_backward, double* loss);
/* Predicted accelerations of the loaded sample, out[n][4] in state order. */
WC_API wc_status wc_surrogate_predictions(wc_surrogate* s, float* out, uint32_t n);
/* One Adam step (beta 0.9 / 0.999, eps 1e-8) with gradients multiplied by grad_scale first;
   clears the accumulated gradients. */
WC_API wc_status wc_surrogate_adam(wc_surrogate* s, float lr, float grad_scale);

typedef struct wc_rollout_stats {
    uint32_t steps, sph_steps, surrogate_steps, judged, reverted;
    uint32_t reserved;
    double mean_density_error; /* mean over judged steps of mean_i |rho_sur_i / rho_sph_i - 1| */
    double max_density_error;
    double ms_device;          /* CUDA-event time of the whole rollout */
    double ms_wall;
    double particle_steps_per_s;
    double diag_start[6];      /* mass, momentum x/y/z, kinetic, potential energy (FP64) */
    double diag_end[6];
} wc_rollout_stats;

/* Rollout modes. SPH: plain solver steps (graph replays). SURROGATE: the network advances the
   fluid. STALE: the method without the network, which reuses the last SPH acceleration for
   the skipped steps (its first step is a plain SPH step that records one). */
#define WC_ROLLOUT_SPH 0
#define WC_ROLLOUT_SURROGATE 1
#define WC_ROLLOUT_STALE 2
/* HYBRID: as STALE, but the skipped steps take the last SPH acceleration plus the network's
   residual, computed with that acceleration and its age as inputs. */
#define WC_ROLLOUT_HYBRID 3

/* Advance the fluid nsteps in `mode`. In the SURROGATE, STALE and HYBRID modes every K-th step
   is judged: SPH and the candidate both advance the same state, the SPH densities of the two next
   states are compared particle by particle, and the SPH state is kept (the step is reverted)
   when the mean |rho_candidate / rho_SPH - 1| exceeds `tolerance`. s may be NULL for SPH.
   hist (host, [5][n][4] in state order, as for wc_surrogate_sample) seeds the surrogate's
   velocity history; NULL starts it as five copies of the current velocity. */
WC_API wc_status wc_surrogate_rollout(wc_surrogate* s, wc_fluid* f, float dt, uint32_t nsteps, uint32_t K,
                                      float tolerance, int mode, const float* hist, wc_rollout_stats* stats);

/* ---- learned fast rollout (no counterpart in the reference) ------------------------------ */
/*
 * Every K-th step is a plain SPH step (the judge); its density pass also computes each
 * particle's density and pressure rates, and its force pass the time derivative J of the SPH
 * acceleration (the pair terms' derivatives under the particles' motion, with the neighbours'
 * density and pressure rates; the viscosity term's neighbour-acceleration part and the wall
 * terms' derivatives are left out). The K-1 skipped steps integrate a(t) + change_k without
 * sorting, where change_k for the step k steps after the judge is, by mode:
 *   WC_LOCAL_STALE    0 (the judge's acceleration held),
 *   WC_LOCAL_TAYLOR   k dt J (first-order extrapolation),
 *   WC_LOCAL_NETWORK  k dt J + the network's residual: a per-particle network maps 19 inputs
 *                     (the SPH acceleration, J x 1 ms, the density rate, velocity, density,
 *                     pressure, six wall distances, k / rho0) through two hidden layers of 64
 *                     (ReLU) to the residuals of ages 1 .. K-1 in units of
 *                     accel_scale (dt / 1 ms)^2, on the tensor cores (BF16 operands, FP32
 *                     accumulation in tensor memory); their mean over the particles is removed.
 * The skipped steps carry each particle's density by its rate. The judge compares that carried
 * density with the SPH density the next judge step computes for the same particles; a cycle
 * whose mean |rho_carried / rho_SPH - 1| exceeds the tolerance is reverted: its K-1 steps are
 * recomputed by plain SPH from the state after the previous judge step.
 */
#define WC_LOCAL_STALE 0
#define WC_LOCAL_TAYLOR 1
#define WC_LOCAL_NETWORK 2
typedef struct wc_local wc_local;

typedef struct wc_local_config {
    uint32_t ages;        /* K - 1: predicted ages, 1 .. 5 */
    uint32_t seed;        /* weight initialisation */
    float accel_scale;    /* accelerations are learned in units of this (m/s^2) */
    float velocity_scale; /* velocities enter in units of this (m/s) */
    uint64_t capacity;    /* training samples kept on the device (rows) */
} wc_local_config;

WC_API void wc_local_config_default(wc_local_config* c);
WC_API wc_status wc_local_create(const wc_local_config* c, wc_local** out);
WC_API void wc_local_destroy(wc_local* net);
WC_API uint64_t wc_local_num_params(const wc_local* net);
WC_API wc_status wc_local_get_params(wc_local* net, float* out, uint64_t count);
WC_API wc_status wc_local_set_params(wc_local* net, const float* in, uint64_t count);
/* Record training samples from `cycles` cycles of plain SPH on a fluid (needs
   WC_FLAG_TRACK_IDS) or a batch: at each cycle's first step the inputs, then the SPH
   accelerations of the next `ages` steps, matched by particle id. The fluid or batch advances
   (ages + 1) * cycles steps. Samples go to the training set, or to the held-out set. */
WC_API wc_status wc_local_record_fluid(wc_local* net, wc_fluid* f, float dt, uint32_t cycles, int held_out);
WC_API wc_status wc_local_record_batch(wc_local* net, wc_batch* b, float dt, uint32_t cycles, int held_out);
WC_API uint64_t wc_local_num_samples(const wc_local* net, int held_out);
WC_API wc_status wc_local_clear_samples(wc_local* net);
/* Adam on the mean squared error over the predicted ages, minibatches of `rows` training samples
   drawn with a fixed generator; loss (optional, host [steps]) gets each step's loss. */
WC_API wc_status wc_local_train(wc_local* net, uint32_t steps, uint32_t rows, float lr, float* loss);
/* Test hook: the loss and the gradient of every parameter ([wc_local_num_params]) on the
   training samples with the given row indices (modulo the sample count), without an update. */
WC_API wc_status wc_local_gradients(wc_local* net, const uint32_t* rows_idx, uint32_t rows, float* grads, float* loss);
/* Copy samples [first, first + count) of a set: inputs [count][32] and targets [count][20]:
   columns 3 (k - 1) .. + 2 the residual (a(t + k) - a(t) - k dt J) / accel_scale of age k,
   column 16 (1 ms / dt)^2 (the residuals' factor into the network's units), columns 17 .. 19
   dt J / accel_scale; either pointer may be NULL. */
WC_API wc_status wc_local_get_samples(wc_local* net, int held_out, uint64_t first, uint64_t count, float* inputs,
                                      float* targets);
/* Relative L2 error of the acceleration at each age over a sample set, host [ages] each, as
   predicted by the network mode, the stale mode and the Taylor mode (err_taylor may be NULL). */
WC_API wc_status wc_local_evaluate(wc_local* net, int held_out, float* err_net, float* err_stale, float* err_taylor);
/* The network's outputs (the residuals of the acceleration changes, [n][3 * ages] floats, host)
   for the fluid's current state: one judge step's inputs without advancing it (test hook of the
   inference). */
WC_API wc_status wc_local_predict(wc_local* net, wc_fluid* f, float dt, float* inputs, float* outputs);
/* Advance the fluid nsteps as cycles of one judge SPH step and `ages` steps in `mode`
   (WC_LOCAL_*; net may be NULL except for WC_LOCAL_NETWORK). */
WC_API wc_status wc_local_rollout_mode(wc_local* net, wc_fluid* f, float dt, uint32_t nsteps, uint32_t ages,
                                       float tolerance, int mode, wc_rollout_stats* stats);
/* wc_local_rollout_mode with WC_LOCAL_NETWORK, or WC_LOCAL_STALE when net is NULL. */
WC_API wc_status wc_local_rollout(wc_local* net, wc_fluid* f, float dt, uint32_t nsteps, uint32_t ages,
                                  float tolerance, wc_rollout_stats* stats);

/* ---- cell sort without allocation ------------------------------------------------------ */

#define WC_NOALLOC_MAX_PARTICLES (1u << 18) /* 262,144 */
#define WC_NOALLOC_MAX_CELLS (1u << 18)     /* grid_res^3 <= 262,144, i.e. grid_res <= 64 */

/*
 * No counterpart in the reference. The cell sort of wc_fluid_sort (keys, stable permutation,
 * cell table, positions gathered into sorted order) as one call that allocates no memory, for
 * callers that cannot allocate when they sort: a frame loop where cudaMalloc would synchronise
 * the GPU, or a host application that fixes its device memory budget up front. Its scratch is
 * one fixed device array (about 4 MB) held by every GPU that loads the library, so it accepts
 * at most WC_NOALLOC_MAX_PARTICLES particles and WC_NOALLOC_MAX_CELLS cells and rejects more
 * with WC_ERR_INVALID_ARG. All buffers are device memory the caller owns:
 *   d_positions        float4[n] (x, y, z, anything)        input
 *   d_keys             uint32[n]   cell key per input particle
 *   d_permutation      uint32[n]   sorted slot -> input index
 *   d_cell_start       uint32[grid_res^3 + 1]  cell c holds slots [start[c], start[c+1])
 *   d_sorted_positions float4[n]   positions in sorted order
 * Work is enqueued on `stream` (a cudaStream_t; NULL = default stream) and not waited for. The
 * first call on a device looks up the array's address and should come before any stream capture.
 * Calls share the array: calls that overlap on the GPU race, so order them on one stream.
 * Device-side errors are not returned by this call (it does not wait); see
 * wc_sort_cells_noalloc_status.
 */
WC_API wc_status wc_sort_cells_noalloc(const void* d_positions, uint32_t n, uint32_t grid_res, float bin_size,
                                       uint32_t* d_keys, uint32_t* d_permutation, uint32_t* d_cell_start,
                                       void* d_sorted_positions, void* stream);

/*
 * No counterpart in the reference. Waits for `stream` and reports the device-side errors of the
 * last wc_sort_cells_noalloc call on the current device, without allocating: WC_ERR_TIMEOUT when
 * a scan tile gave up waiting (that call's cell table and permutation are invalid),
 * WC_ERR_NUMERIC for a non-finite position (binned to cell 0) or a cell of more than 65,536
 * particles (its members are placed in arrival order, not input order), else WC_OK.
 */
WC_API wc_status wc_sort_cells_noalloc_status(void* stream);

/* Make `device` current for handles created afterwards on this thread (one process per GPU). */
/* Test hook, not for production use: with on != 0 the cell scan's look-back polls a descriptor
   that nothing publishes, so every scan tile after the first gives up after spin_limit polls and
   the step reports WC_ERR_TIMEOUT (the tables of that step are invalid, every access stays in
   bounds); on = 0 restores normal operation. Applies to the current device, for all handles. */
WC_API wc_status wc_debug_scan_stall(int on, uint32_t spin_limit);
/* Test hook, not for production use: after `after` more successful device allocations, every
   allocation the library makes fails with WC_ERR_OOM (its callers unwind and free what they
   hold); after < 0 switches the hook off. Process-wide. */
WC_API void wc_debug_fail_allocations(long long after);

WC_API wc_status wc_set_device(int device);
WC_API int wc_device_count(void);

/* Page-locked host memory for the host copies (faster and asynchronous-capable transfers). */
WC_API wc_status wc_alloc_host(size_t bytes, void** out);
WC_API void wc_free_host(void* p);

/* ---- errors and build info -------------------------------------------------------------- */

/* Message of the last failing call on this thread ("" if none). */
WC_API const char* wc_last_error(void);
WC_API const char* wc_status_string(wc_status s);
/* e.g. "watercube 1 sm_103a" */
WC_API const char* wc_build_info(void);

#ifdef __cplusplus
}
#endif

#endif /* WATERCUBE_H */

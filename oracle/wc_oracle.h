/*
 * wc_oracle.h — CPU oracle for the SPH solver. TEST INFRASTRUCTURE ONLY: the test suite, the
 * smoke check and bench.py's CPU-baseline leg are its only users; the solver never calls it.
 *
 * It restates WaterCube's particle pipeline on the host, stage by stage:
 *   wco_sort          assets/sort/count.comp:25-36, linearScan.comp:15-28, reorder.comp:32-45,
 *                     sort.comp:32-45, in the order of Sort::run (src/core/Sort.cpp:254-267)
 *   wco_density_*     assets/fluid/density.comp:52-137
 *   wco_update_*      assets/fluid/update.comp:61-232
 *   wco_step_*        Fluid::update (src/core/Fluid.cpp:342-354)
 * The float path repeats the shaders' float operations in their order (so that, with the
 * built-in semantics stated in wc_oracle.cpp, it equals the shaders compiled as C++ bit for
 * bit); the double path evaluates the same equations in FP64 and is the tolerance oracle.
 *
 * Parity pin: oracle/ref/make_ref.py compiles the reference's own compute shaders as C++
 * into oracle/_ref/; tests/test_oracle_ref.py and the committed fixtures in tests/golden/
 * (made by tests/golden/make_golden.py from that build) check this restatement against it.
 */
#ifndef WC_ORACLE_H
#define WC_ORACLE_H

#include <stdint.h>

#include "../include/watercube.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct wco_particle64 {
    double position[3];
    double density;
    double velocity[3];
    double pressure;
} wco_particle64;

/* FP64 scene diagnostics: total mass, momentum, kinetic and potential (m g.y... = -m g.x) energy. */
typedef struct wco_diagnostics {
    double mass;
    double momentum[3];
    double kinetic;
    double potential;
} wco_diagnostics;

/* Stable counting sort by cell key. counts/offsets have grid_res^3 entries; out/keys/perm n. */
int wco_sort(const wc_params* p, const wc_particle* in, uint32_t n, wc_particle* out, uint32_t* keys,
             uint32_t* perm, uint32_t* counts, uint32_t* offsets);
int wco_sort64(const wc_params* p, const wco_particle64* in, uint32_t n, wco_particle64* out, uint32_t* keys,
               uint32_t* perm, uint32_t* counts, uint32_t* offsets);

/* Density + pressure in place on a sorted buffer. ncount (optional) gets per-particle neighbour
   counts (j != i, |r| < h). */
int wco_density_f32(const wc_params* p, wc_particle* sorted, uint32_t n, const uint32_t* counts,
                    const uint32_t* offsets, uint32_t* ncount, int threads);
int wco_density_f64(const wc_params* p, wco_particle64* sorted, uint32_t n, const uint32_t* counts,
                    const uint32_t* offsets, uint32_t* ncount, int threads);

/* Forces + symplectic Euler + wall collision: in (sorted) -> out (same order). */
int wco_update_f32(const wc_params* p, const wc_particle* in, wc_particle* out, uint32_t n, const uint32_t* counts,
                   const uint32_t* offsets, float dt, int threads);
int wco_update_f64(const wc_params* p, const wco_particle64* in, wco_particle64* out, uint32_t n,
                   const uint32_t* counts, const uint32_t* offsets, double dt, int threads);

/* nsteps full updates (sort, density, update); the state stays in sorted order, as the
   reference leaves it. ids (optional) is permuted along with the particles. */
int wco_step_f32(const wc_params* p, wc_particle* state, uint32_t n, float dt, uint32_t nsteps, uint32_t* ids,
                 int threads);
int wco_step_f64(const wc_params* p, wco_particle64* state, uint32_t n, double dt, uint32_t nsteps, uint32_t* ids,
                 int threads);

/* Initial states; same definitions as wc_generate_* in the solver's header. */
int wco_generate_dam_break(const wc_params* p, uint64_t seed, wc_particle* out, uint32_t n);
int wco_generate_reference_lattice(const wc_params* p, uint64_t seed, wc_particle* out, uint32_t n);

/* Parameters without the solver library: the dam-break preset and Fluid::setup's derivation
   (src/core/Fluid.cpp:207-216); the same values as wc_params_dam_break / wc_params_finalize. */
int wco_params_dam_break(wc_params* p, uint32_t n);
int wco_params_finalize(wc_params* p);

int wco_diagnostics_f32(const wc_params* p, const wc_particle* s, uint32_t n, wco_diagnostics* out);
int wco_diagnostics_f64(const wc_params* p, const wco_particle64* s, uint32_t n, wco_diagnostics* out);

/* Largest float x with sqrtf(x) < h, found by stepping through floats around h*h. */
float wco_cull_threshold(float h);

int wco_max_threads(void);

#ifdef __cplusplus
}
#endif

#endif

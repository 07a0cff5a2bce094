// ref_driver.cpp — host driver for the reference's compute shaders compiled as C++ (see
// make_ref.py). TEST INFRASTRUCTURE ONLY: it builds the parity reference and the reference arm
// of the benchmark, never the solver.
//
// It replays the reference's dispatch sequence with the same uniforms:
//   wcref_sort   = Sort::run            (src/core/Sort.cpp:254-267, uniforms :168-213)
//   wcref_perm   = Sort::runSortProg    (src/core/Sort.cpp:218-232; compiled but never dispatched
//                                        by the reference — it specifies the permutation output)
//   wcref_density= Fluid::runDensityProg (src/core/Fluid.cpp:268-289)
//   wcref_update = Fluid::runUpdateProg  (src/core/Fluid.cpp:294-321)
//   wcref_step   = Fluid::update         (src/core/Fluid.cpp:342-354)
// A dispatch of G work groups runs invocations 0 .. G*local_size-1 (util::runProg,
// src/core/util.cpp:32-36); with threads == 1 they run in id order, so the atomicAdd ranks of
// reorder.comp come out stable.
#include <cstdint>
#include <cstring>

#include "../../include/watercube.h"
#include "glsl_compat.h"

thread_local glsl::uvec3 gl_GlobalInvocationID;

#define WCREF_DECL(S)                                                                     \
    extern "C" int wcref_##S##_set_buffer(const char* name, void* ptr);                   \
    extern "C" int wcref_##S##_set_float(const char* name, const float* v, int n);        \
    extern "C" int wcref_##S##_set_int(const char* name, int v);                          \
    extern "C" void wcref_##S##_dispatch(unsigned groups, int threads);                   \
    extern "C" unsigned wcref_##S##_local_size(void);
WCREF_DECL(count)
WCREF_DECL(linearScan)
WCREF_DECL(reorder)
WCREF_DECL(sort)
WCREF_DECL(density)
WCREF_DECL(update)

namespace {

int g_bad = 0;
void req(int rc) { g_bad |= (rc != 0); }

unsigned groups_for(unsigned n, unsigned local) { return (n + local - 1) / local; }

void clear(uint32_t* buf, uint32_t C) { std::memset(buf, 0, sizeof(uint32_t) * C); }

}  // namespace

extern "C" {

int wcref_sort(const wc_params* p, wc_particle* in, wc_particle* out, uint32_t* counts, uint32_t* offsets,
               uint32_t n, int threads) {
    g_bad = 0;
    const uint32_t R = p->grid_res, C = R * R * R;
    const int gr = (int)R, ni = (int)n;
    clear(counts, C);  // clearCountBuffer
    req(wcref_count_set_buffer("particles", in));
    req(wcref_count_set_buffer("counts", counts));
    req(wcref_count_set_float("binSize", &p->bin_size, 1));
    req(wcref_count_set_int("numItems", ni));
    req(wcref_count_set_int("gridRes", gr));
    if (g_bad) return -1;
    wcref_count_dispatch(groups_for(n, wcref_count_local_size()), threads);

    clear(offsets, C);  // clearOffsetBuffer
    req(wcref_linearScan_set_buffer("counts", counts));
    req(wcref_linearScan_set_buffer("offsets", offsets));
    req(wcref_linearScan_set_int("gridRes", gr));
    if (g_bad) return -1;
    wcref_linearScan_dispatch(1, 1);  // a single invocation (Sort.cpp:192)

    clear(counts, C);  // clearCountBuffer
    req(wcref_reorder_set_buffer("inParticles", in));
    req(wcref_reorder_set_buffer("outParticles", out));
    req(wcref_reorder_set_buffer("counts", counts));
    req(wcref_reorder_set_buffer("offsets", offsets));
    req(wcref_reorder_set_float("binSize", &p->bin_size, 1));
    req(wcref_reorder_set_int("numItems", ni));
    req(wcref_reorder_set_int("gridRes", gr));
    if (g_bad) return -1;
    wcref_reorder_dispatch(groups_for(n, wcref_reorder_local_size()), threads);
    return 0;
}

// sort.comp over the same input: needs offsets from wcref_sort; leaves counts as the histogram.
int wcref_perm(const wc_params* p, wc_particle* in, uint32_t* counts, uint32_t* offsets, uint32_t* sorted,
               uint32_t n, int threads) {
    g_bad = 0;
    const uint32_t R = p->grid_res, C = R * R * R;
    clear(counts, C);
    req(wcref_sort_set_buffer("particles", in));
    req(wcref_sort_set_buffer("counts", counts));
    req(wcref_sort_set_buffer("offsets", offsets));
    req(wcref_sort_set_buffer("sorted", sorted));
    req(wcref_sort_set_float("binSize", &p->bin_size, 1));
    req(wcref_sort_set_int("numItems", (int)n));
    req(wcref_sort_set_int("gridRes", (int)R));
    if (g_bad) return -1;
    wcref_sort_dispatch(groups_for(n, wcref_sort_local_size()), threads);
    return 0;
}

int wcref_density(const wc_params* p, wc_particle* particles, uint32_t* counts, uint32_t* offsets, uint32_t* debug,
                  uint32_t n, int threads) {
    g_bad = 0;
    req(wcref_density_set_buffer("particles", particles));
    req(wcref_density_set_buffer("counts", counts));
    req(wcref_density_set_buffer("offsets", offsets));
    req(wcref_density_set_buffer("debug", debug));
    req(wcref_density_set_float("size", &p->size, 1));
    req(wcref_density_set_float("binSize", &p->bin_size, 1));
    req(wcref_density_set_int("gridRes", (int)p->grid_res));
    req(wcref_density_set_int("numParticles", (int)n));
    req(wcref_density_set_float("particleMass", &p->particle_mass, 1));
    req(wcref_density_set_float("kernelRadius", &p->kernel_radius, 1));
    req(wcref_density_set_float("stiffness", &p->stiffness, 1));
    req(wcref_density_set_float("restDensity", &p->rest_density, 1));
    req(wcref_density_set_float("restPressure", &p->rest_pressure, 1));
    req(wcref_density_set_float("poly6KernelConst", &p->poly6_const, 1));
    if (g_bad) return -1;
    wcref_density_dispatch(groups_for(n, wcref_density_local_size()), threads);
    return 0;
}

int wcref_update(const wc_params* p, wc_particle* in, wc_particle* out, uint32_t* counts, uint32_t* offsets,
                 uint32_t* debug, uint32_t n, float dt, int threads) {
    g_bad = 0;
    req(wcref_update_set_buffer("inParticles", in));
    req(wcref_update_set_buffer("outParticles", out));
    req(wcref_update_set_buffer("counts", counts));
    req(wcref_update_set_buffer("offsets", offsets));
    req(wcref_update_set_buffer("debug", debug));
    req(wcref_update_set_float("size", &p->size, 1));
    req(wcref_update_set_float("binSize", &p->bin_size, 1));
    req(wcref_update_set_int("gridRes", (int)p->grid_res));
    req(wcref_update_set_float("dt", &dt, 1));
    req(wcref_update_set_int("numParticles", (int)n));
    req(wcref_update_set_float("gravity", p->gravity, 3));
    req(wcref_update_set_float("particleMass", &p->particle_mass, 1));
    req(wcref_update_set_float("kernelRadius", &p->kernel_radius, 1));
    req(wcref_update_set_float("viscosityCoefficient", &p->viscosity, 1));
    req(wcref_update_set_float("cameraPosition", p->mouse_origin, 3));
    req(wcref_update_set_float("mouseRayDirection", p->mouse_dir, 3));
    req(wcref_update_set_float("spikyKernelConst", &p->spiky_const, 1));
    req(wcref_update_set_float("viscosityKernelConst", &p->visc_const, 1));
    if (g_bad) return -1;
    wcref_update_dispatch(groups_for(n, wcref_update_local_size()), threads);
    return 0;
}

// Fluid::update: sort buf1 -> buf2, density on buf2, update buf2 -> buf1; nsteps times.
int wcref_step(const wc_params* p, wc_particle* buf1, wc_particle* buf2, uint32_t* counts, uint32_t* offsets,
               uint32_t* debug, uint32_t n, float dt, uint32_t nsteps, int threads) {
    for (uint32_t s = 0; s < nsteps; ++s) {
        if (wcref_sort(p, buf1, buf2, counts, offsets, n, threads)) return -1;
        if (wcref_density(p, buf2, counts, offsets, debug, n, threads)) return -1;
        if (wcref_update(p, buf2, buf1, counts, offsets, debug, n, dt, threads)) return -1;
    }
    return 0;
}

}  // extern "C"

// Drives the solver through the C++ drop-in exactly as WaterCubeApp drives core::Fluid
// (src/WaterCubeApp.cpp:58-64, :98): create, chained setters, setup, update per frame.
// Prints "ok <particles> <steps>" and exits 0 when every particle stays finite inside the box.
#include <cmath>
#include <cstdio>
#include <cstring>

#include "watercube/Fluid.hpp"

int main() {
    try {
        core::FluidRef fluid = core::Fluid::create("fluid");
        fluid->numParticles(20000)->gridRes(21)->viscosityCoefficient(200.0f)->stiffness(100.0f);
        fluid->setup();
        const int frames = 30;
        for (int i = 0; i < frames; ++i) fluid->update(1.0 / 60.0);
        const std::vector<wc_particle> p = fluid->particles();
        const std::vector<uint32_t> counts = fluid->uints(WC_UINTS_CELL_COUNTS);
        // one frame with host buffers equals upload + update + readback
        std::vector<wc_particle> stepped(p.size());
        fluid->updateHost(1.0 / 60.0, p.data(), stepped.data());
        if (fluid->particles().size() != stepped.size()) return 1;
        const std::vector<wc_particle> again = fluid->particles();
        for (size_t i = 0; i < again.size(); ++i)
            if (std::memcmp(&again[i], &stepped[i], sizeof(wc_particle)) != 0) {
                std::printf("updateHost readback differs from particles() at %zu\n", i);
                return 1;
            }
        fluid->synchronize();
        uint64_t total = 0;
        for (uint32_t c : counts) total += c;
        if (total != p.size()) {
            std::printf("cell counts sum %llu != %zu\n", (unsigned long long)total, p.size());
            return 1;
        }
        for (const wc_particle& q : p)
            for (int a = 0; a < 3; ++a)
                if (!std::isfinite(q.position[a]) || q.position[a] < 0.0f || q.position[a] > 1.0f) {
                    std::printf("particle outside the box\n");
                    return 1;
                }
        bool threw = false;
        try {
            fluid->numParticles(10);  // parameters are fixed after setup
        } catch (const core::FluidError& e) {
            threw = e.status == WC_ERR_STATE;
        }
        if (!threw) return 1;
        std::printf("ok %zu %d\n", p.size(), frames);
        return 0;
    } catch (const std::exception& e) {
        std::printf("error: %s\n", e.what());
        return 1;
    }
}

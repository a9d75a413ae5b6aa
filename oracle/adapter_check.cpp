// adapter_check.cpp -- compiles GpuForceCalculation against the reference's
// own headers and hands it to the reference's LeapfrogDKD as its
// ForceCalculationMethod&.  Built by `make -C oracle adapter` (links the
// reference objects of oracle/_ref/stock and libsolveit_gpu.so).  Running it
// needs a GPU; the CPU tests only build it, which is what proves the adapter
// is a drop-in for the reference's interface.
#include "force_calculation_methods.h"
#include "integration_schemes.h"
#include "../solveit-code_gb300/adapter/gpu_force_calculation.h"

int main(int argc, char **argv) {
    const int n = argc > 1 ? std::atoi(argv[1]) : 256;
    ParticleSystem ps;
    ChargedParticles &cp = ps.chargedParticles;
    cp.allocateMemory(n);
    for (int i = 0; i < n; i++) {
        cp.position[i] = vec4<float>(1e-9f * (i % 7), 1e-9f * (i % 5), 1e-9f * i, 1.0f);
        cp.velocity[i] = vec4<float>(0.0f, 0.0f, 2e4f, (float)(i & 1));
        cp.acceleration[i] = vec4<float>(0.0f, 0.0f, 0.0f, 1.0f);
        cp.timeInjected[i] = 0.0f;
        cp.Efield1[i] = 0.0f;
        cp.Efield2[i] = 0.0f;
    }
    cp.firstParticle = 0;
    cp.lastParticle = n;
    GpuForceCalculation gpu(&ps, SV_METHOD_FMM);
    gpu.setNumExpansions(8);
    gpu.setWellSeparation(2);
    ForceCalculationMethod &fm = gpu;
    LeapfrogDKD leap(ps, fm);  // the reference integrator accepts the adapter as its force method
    (void)leap;
    fm.setFirstParticle(0);
    fm.setLastParticle(n);
    fm.updateAcceleration();
    std::printf("a[0] = %g %g %g\n", cp.acceleration[0].x, cp.acceleration[0].y, cp.acceleration[0].z);
    std::fflush(nullptr);
    std::_Exit(0);
}

// gpu_force_calculation.h -- the GB300 engine as a SOLVEiT ForceCalculationMethod.
//
// Drop-in for DirectForceCalculation / BarnesHutForceCalculation /
// MultipoleMethodForceCalculation (force_calculation_methods.h:28-87): an
// integrator holding a ForceCalculationMethod& (integration_schemes.h:21-87)
// drives it unchanged.  updateAcceleration() keeps the reference contract:
// for i in [firstParticle, lastParticle) with acceleration[i].w == inbound it
// ADDS the particle-particle acceleration (m/s^2) into acceleration[i].xyz;
// sources are the particles of that range with w in {inbound,
// affectsAcceleration}; the arrays keep their order.  The symmetry variant
// follows particleSystem->params.symType, the periodic images setGrid() /
// params.domainSize, exactly as the reference methods read them.
//
// Header-only; compile together with the reference headers and link
// libsolveit_gpu.so.  The reference's own FP32 vec4 arrays are uploaded as they
// are (positions widened to FP64 on the device, masses from the species code).
#pragma once

#include <cstdio>
#include <cstdlib>

#include "force_calculation_methods.h"
#include "solveit_gpu.h"

class GpuForceCalculation : public ForceCalculationMethod {
public:
    explicit GpuForceCalculation(ParticleSystem *particleSystem, sv_method method = SV_METHOD_DIRECT,
                                 sv_precision precision = SV_PREC_MIXED)
        : ForceCalculationMethod{particleSystem} {
        sv_default_params(&params_);
        params_.method = method;
        params_.precision = precision;
        params_.softening2 = PhysicalConstant::SOFTENING;
        params_.k_const = PhysicalConstant::K_CONST;
        setTimerName();
        setSaveName();
    }
    ~GpuForceCalculation() { sv_destroy(ctx_); }

    // setTheta (barnes_hut_force_calculation.cpp:110), setNumExpansions, ...
    void setTheta(float theta) { params_.theta = theta; }
    void setNumExpansions(int p) { params_.fmm_order = p; }
    void setWellSeparation(int ws) { params_.fmm_ws = ws; }
    void setLeafSize(int n) { params_.leaf_size = n; }
    void setSoftening(double eps2) { params_.softening2 = eps2; }
    void setDevice(int device) { params_.device = device; }
    // the FmmType the reference passes to MultipoleMethodForceCalculation's
    // constructor (multipole_method_force_calculation.cpp:9-104)
    void setFmmType(sv_fmm_type t) { params_.fmm_type = t; }
    // the FMM root cube's scale (sv_params.fmm_root_scale), or sv_fmm_tune on
    // the first evaluation's state when autoTune is set
    void setRootScale(float s) { params_.fmm_root_scale = s; }
    void setAutoTune(bool on) {
        autoTune_ = on;
        tuned_ = false;
    }

    void updateAcceleration() override {
        if (particleSystem == nullptr) {
            printf("Particle system not initialized.\n");
            exit(1);
        }
        const int n = lastParticle - firstParticle;
        if (n <= 0) return;
        syncSymmetry();
        if (ctx_ == nullptr) {
            check(sv_create(&params_, &ctx_), "sv_create");
        } else {
            check(sv_set_params(ctx_, &params_), "sv_set_params");
        }
        ChargedParticles &cp = particleSystem->chargedParticles;
        const int f = firstParticle;
        check(sv_upload_ref32(ctx_, n, &cp.position[f].x, &cp.velocity[f].x, &cp.acceleration[f].x,
                              cp.timeInjected ? &cp.timeInjected[f] : nullptr),
              "sv_upload_ref32");
        if (autoTune_ && !tuned_ && params_.method == SV_METHOD_FMM) {
            check(sv_fmm_tune(ctx_, nullptr), "sv_fmm_tune");
            check(sv_get_params(ctx_, &params_), "sv_get_params");  // keeps the tuned scale
            tuned_ = true;
        }
        check(sv_compute_accel(ctx_, 0, n, nullptr), "sv_compute_accel");
        check(sv_add_accel_ref32(ctx_, &cp.acceleration[f].x), "sv_add_accel_ref32");
        if (timeInfoFile != nullptr) {
            sv_stats st;
            sv_get_stats(ctx_, &st);
            const float ms = (float)st.ms_total;
            fwrite(&n, sizeof(n), 1, timeInfoFile);
            fwrite(&ms, sizeof(ms), 1, timeInfoFile);
        }
    }

    // the reference's integrator calls this when a deeper FMM level measured
    // faster (Integrator::compareAcceleration): tune the root scale again at
    // the next evaluation
    void increaseLevel() override { tuned_ = false; }
    void setSaveName() override {
        if (saveName[0] == '\0') saveName = "_gpu.bin";
    }
    void setTimerName() override {
        if (timerName[0] == '\0') timerName = "GB300 Force Method";
    }

protected:
    void allocateThreadMemory() override {}
    void deallocateThreadMemory() override {}

private:
    void syncSymmetry() {
        const SimulationParameters &sp = particleSystem->params;
        switch (sp.symType) {
        case SymmetryType::rotational: params_.symmetry = SV_SYM_ROTATIONAL; break;
        case SymmetryType::translational: params_.symmetry = SV_SYM_TRANSLATIONAL; break;
        default: params_.symmetry = SV_SYM_NONE; break;
        }
        if (params_.symmetry == SV_SYM_TRANSLATIONAL) {
            const vec3<int> ax = grid != nullptr ? grid->symmetryAxes : sp.symmetryAxes;
            params_.sym_axes[0] = ax.x;
            params_.sym_axes[1] = ax.y;
            params_.sym_axes[2] = ax.z;
            params_.sym_levels = sp.numSymmetryLevels;
            params_.domain_size[0] = sp.domainSize.x;
            params_.domain_size[1] = sp.domainSize.y;
            params_.domain_size[2] = sp.domainSize.z;
        }
    }
    void check(sv_status s, const char *what) {
        if (s != SV_OK) {
            printf("%s failed (%d): %s\n", what, (int)s, sv_last_error(ctx_));
            exit(1);
        }
    }

    sv_params params_;
    sv_ctx *ctx_ = nullptr;
    bool autoTune_ = false, tuned_ = false;
};

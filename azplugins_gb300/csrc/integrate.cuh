// integrate.cuh -- Langevin / Brownian dynamics in a flow field, device side.
//
// Math of the reference's legacy integrators:
//   step one   src/TwoStepLangevinFlow.h:128-153, GPU src/TwoStepLangevinFlowGPU.cu:19-58
//   step two   src/TwoStepLangevinFlow.h:194-245, GPU src/TwoStepLangevinFlowGPU.cuh:60-147
//   Brownian   src/TwoStepBrownianFlow.h:136-178, GPU src/TwoStepBrownianFlowGPU.cuh:50-127
// One difference on purpose: the Brownian step keeps the type bits of pos.w
// (the reference writes the type as a number, src/TwoStepBrownianFlow.h:177).
#pragma once

#include "common.cuh"
#include "philox.cuh"

namespace azp
{
constexpr uint32_t MAX_GAMMA_TYPES = 64;

// Flow fields (src/ConstantFlow.h:48-51, src/ParabolicFlow.h:69-93).
struct FlowD {
    int kind;
    double a, b, c;  // CONSTANT: U; PARABOLIC: a = Umax = 1.5 mean_velocity, b = L = separation / 2
};

inline FlowD make_flow(const azp_flow& f)
{
    FlowD r;
    r.kind = f.kind;
    if (f.kind == AZP_FLOW_PARABOLIC) {
        r.a = 1.5 * f.p[0];
        r.b = 0.5 * f.p[1];
        r.c = 0.0;
    } else {
        r.a = f.p[0];
        r.b = f.p[1];
        r.c = f.p[2];
    }
    return r;
}

AZP_D void flow_at(const FlowD& f, double y, double& ux, double& uy, double& uz)
{
    if (f.kind == AZP_FLOW_PARABOLIC) {
        const double yr = y / f.b;
        ux = f.a * (1.0 - yr * yr);
        uy = 0.0;
        uz = 0.0;
    } else {
        ux = f.a;
        uy = f.b;
        uz = f.c;
    }
}

// flow field in FP32 (same functor values to FP32 rounding)
AZP_D void flow_at_f(const FlowD& f, float y, float& ux, float& uy, float& uz)
{
    if (f.kind == AZP_FLOW_PARABOLIC) {
        const float yr = y * (float)(1.0 / f.b);
        ux = (float)f.a * (1.0f - yr * yr);
        uy = 0.0f;
        uz = 0.0f;
    } else {
        ux = (float)f.a;
        uy = (float)f.b;
        uz = (float)f.c;
    }
}

AZP_D void wrap1(double& x, int& img, double L, double lo, double hi)
{
    if (x >= hi) {
        x -= L;
        img += 1;
    } else if (x < lo) {
        x += L;
        img -= 1;
    }
}

struct StepArgs {
    double4_32a* pos;
    double4_32a* vel;
    double* accel;      // [N][3]
    int* image;         // [N][3]
    const uint32_t* tag;
    const double* diameter;
    const uint32_t* group;
    uint32_t n;
    double L[3], lo[3], hi[3];
    double dt, kT;
    uint64_t timestep;
    uint32_t seed;
    int noiseless;
    const void* net_force;
    int net_precision;
    const double* gamma;  // device [ntypes]
    uint32_t ntypes;
    int use_lambda;
    double lambda;
    FlowD flow;
    double max_disp;
};

int launch_step1(const StepArgs& a, cudaStream_t s);
int launch_step2(const StepArgs& a, cudaStream_t s);
int launch_brownian(const StepArgs& a, cudaStream_t s);
int launch_uniform3(uint32_t id, uint64_t timestep, uint32_t seed, const uint32_t* tags, uint32_t n, double lo,
                    double hi, double* out, cudaStream_t s);

}  // namespace azp

// The learned-lambda network handle, shared by mlp.cu (its C ABI) and pbf_solver.cu (which
// launches the network's forward pass inside the step's graph).
#pragma once

#include <cstdint>

struct akua_mlp {
    int device = 0;
    int sms = 0;
    float* params = nullptr;  // FP32 master parameters [kParams]
    uint8_t* image = nullptr; // BF16 operand images of W1..W3 for the forward pass
    float* grad = nullptr;    // [kParams] gradient, then the loss
    float* m = nullptr;       // Adam moments
    float* v = nullptr;
    float* norm = nullptr;    // mean[8], inv_std[8], out_scale
    uint32_t* err = nullptr;  // device error flags (bit 0: an MMA wait timed out)
    int64_t adam_steps = 0;
};

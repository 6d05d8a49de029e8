// Backward pass of a reconstructed frame (see backward.cu).
#pragma once

#include "kernels.h"

namespace fsr {

struct BwdArgs {
    Grid sp, sc;
    uint32_t ratio;
    uint32_t n;
    BandView band;
    const uint32_t* sv;
    const uint32_t* valid;
    const uint32_t* mc;
    const uint32_t* vofs;
    const uint64_t* tri;     // packed marching-cubes triangle table (device)
    const float* gmesh;      // dL/d mesh vertex positions, 3 floats each
    float* gphi;             // dL/dphi per band vertex (zeroed)
    uint32_t* gkey;          // per window-centre key: holds a vertex with dL/dphi != 0 (zeroed)
    uint32_t* glist;         // [0] keys listed, [1] [2] work counters of the grouped adjoints (zeroed),
                             // [4 ..] the keys with gkey set, in the order k_mark_keys met them
    const float4* sorted;
    const uint32_t* skeys;
    const uint32_t* perm;
    const uint8_t* invol;
    const float4* smoothed;
    const float4* grec;
    const float4* qrec;  // the field's records: (x~, r2max) (M00, 2M01, 2M02, coef) (M11, 2M12, M22, 0)
    const uint2* ranges;
    const float* cell_rmax;  // Yu13: per cell, largest support reach of its particles
    const float4* mv;        // ZB05: per band vertex (mean - v, weight sum)
    float4* gsmooth;         // dL/d smoothed position (Yu13; zeroed); w: sum dL/dphi (1 - q2)^3
    float4* gG;              // dL/dG, 3 float4 rows per particle (Yu13; zeroed)
    float4* gmean;           // dL/d mean from the covariance (Yu13)
    float4* gx;              // dL/dx in sorted order (zeroed)
    float iso, h, sigma;
    uint32_t cap_band, cap_valid;
};

// Grouped adjoint of the ZB05 / TC01 fields (field_aniso.cu); adds into a.gx
// (zeroed).  Returns false (nothing launched) when the grid ratio makes a
// group too large for shared memory.
bool launch_field_iso_backward_grouped(const KernelCtx& c, const BwdArgs& a, bool tc01, const Counters* ctr);

void launch_backward(const KernelCtx& c, const BwdArgs& a, const CovArgs* cov, const Counters* ctr, int method,
                     float lambda, float R, float* radius_grad_dev, float* out_grad_xyz);

}  // namespace fsr

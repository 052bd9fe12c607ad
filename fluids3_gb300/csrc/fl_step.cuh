// Per-point arithmetic of the step shared by the neighbour passes
// (fl_kernels.cu, fl_cells.cu): packed FP32 helpers, one pair's force term
// and the advance of one point, each in the reference kernels' own
// operation order. Included
// inside each file's anonymous namespace; both files are compiled without
// FMA contraction, so every expression rounds as written.
#pragma once

// ---- packed f32x2 arithmetic (round-to-nearest per element) ---------------
// Each packed operation rounds exactly like its scalar form, but ptxas
// contracts a packed add of two packed products into a packed fused
// multiply-add (measured on GB300, explicit .rn and --fmad=false
// notwithstanding): no add2 here may take two mul2 results.
__device__ __forceinline__ uint64_t pk2(float a, float b) {
    uint64_t r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void up2(uint64_t v, float &a, float &b) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(v));
}
__device__ __forceinline__ uint64_t add2(uint64_t a, uint64_t b) {
    uint64_t r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ uint64_t sub2(uint64_t a, uint64_t b) {
    uint64_t r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ uint64_t mul2(uint64_t a, uint64_t b) {
    uint64_t r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}


struct ForcePoint {
    float4 p, vi;
    float di, pi;
    float3 f;
};

// One pair's force term on a point at p (pressure term pi, evaluated
// velocity vi, density di) from the neighbour's position q, evaluated
// velocity vj and density dj, in the reference's operation order
// (fluid_kernels.cu:203-210); the pair is known to pass 0 < d^2 < rd2. The
// point's force is the sum of its terms, added component-wise in the
// reference's pair order.
__device__ __forceinline__ float3 pair_term(const DevParams &P, float4 p, float pi, float4 vi, float di, float4 q,
                                            float4 vj, float dj) {
    const float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
    const float dsq = dx * dx + dy * dy + dz * dz;
    const float r = sqrtf(dsq * P.d2);
    const float pj = (dj - P.prest_dens) * P.pintstiff;
    const float cr = P.psmoothradius - r;
    const float pterm = P.sim_scale * -0.5f * cr * P.spikykern * (pi + pj) / r;
    const float sx = dx * pterm + (vj.x - vi.x) * P.vterm;
    const float sy = dy * pterm + (vj.y - vi.y) * P.vterm;
    const float sz = dz * pterm + (vj.z - vi.z) * P.vterm;
    const float inv = 1.0f / (di * dj);
    return make_float3((sx * cr) * inv, (sy * cr) * inv, (sz * cr) * inv);
}

__device__ __forceinline__ void add_pair_terms(const DevParams &P, ForcePoint &fp, float4 q, float4 vj,
                                               float dj) {
    const float3 t = pair_term(P, fp.p, fp.pi, fp.vi, fp.di, q, vj, dj);
    fp.f.x += t.x;
    fp.f.y += t.y;
    fp.f.z += t.z;
}

// advanceParticles body (fluids4.0/fluid_kernels.cu:343-419) for an
// in-range point: walls, gravity, limits, leapfrog. `accel` enters as the
// SPH force; returns the new position, velocity and evaluated velocity.
__device__ __forceinline__ void advance_point(const DevParams &P, float time, float dt, float ss,
                                              float3 accel, float3 pos, float3 vel, float3 veval,
                                              float3 &pos_o, float3 &vel_o, float3 &veval_o) {
    accel.x *= P.pmass; accel.y *= P.pmass; accel.z *= P.pmass;
    float diff, adj;
    // Y- wall with slope (cu:356-361)
    diff = P.pradius - (pos.y - (P.bound_min.y + (pos.x - P.bound_min.x) * P.bound_slope)) * ss;
    if (diff > kEpsilon) {
        float3 nrm = make_float3(-P.bound_slope, 1.0f - P.bound_slope, 0.0f);
        adj = P.bound_stiff * diff - P.bound_damp * (nrm.x * veval.x + nrm.y * veval.y + nrm.z * veval.z);
        nrm.x *= adj; nrm.y *= adj; nrm.z *= adj;
        accel.x += nrm.x - veval.x * P.bound_friction;
        accel.y += nrm.y - veval.y * P.bound_friction;
        accel.z += nrm.z - veval.z * P.bound_friction;
    }
    // Y+ (cu:363-368)
    diff = P.pradius - (P.bound_max.y - pos.y) * ss;
    if (diff > kEpsilon) {
        float3 nrm = make_float3(0.0f, -1.0f, 0.0f);
        adj = P.bound_stiff * diff - P.bound_damp * (nrm.x * veval.x + nrm.y * veval.y + nrm.z * veval.z);
        nrm.x *= adj; nrm.y *= adj; nrm.z *= adj;
        accel.x += nrm.x - veval.x * P.bound_friction;
        accel.y += nrm.y - veval.y * P.bound_friction;
        accel.z += nrm.z - veval.z * P.bound_friction;
    }
    // X- moving wall (cu:371-377): stiffness scaled by the wall term. The
    // reference forms `sin(..) * 0.5 + 0.5` and the amplitude product with
    // double literals, so the product is formed in double and rounded once
    // to float, as there (three FP64 operations per point).
    const float wall = (float)(((double)sinf(time * P.bound_wall_freq + pos.z / 400.f) * 0.5 + 0.5) *
                               (double)P.bound_wall_force);
    diff = P.pradius - (pos.x - (P.bound_min.x + wall)) * ss;
    if (diff > kEpsilon) {
        float3 nrm = make_float3(1.0f, 0.0f, 0.0f);
        adj = wall * P.bound_stiff * diff - P.bound_damp * (nrm.x * veval.x + nrm.y * veval.y + nrm.z * veval.z);
        accel.x += nrm.x * adj; accel.y += nrm.y * adj; accel.z += nrm.z * adj;
    }
    // X+ (cu:378-383)
    diff = P.pradius - (P.bound_max.x - pos.x) * ss;
    if (diff > kEpsilon) {
        float3 nrm = make_float3(-1.0f, 0.0f, 0.0f);
        adj = P.bound_stiff * diff - P.bound_damp * (nrm.x * veval.x + nrm.y * veval.y + nrm.z * veval.z);
        accel.x += nrm.x * adj; accel.y += nrm.y * adj; accel.z += nrm.z * adj;
    }
    // Z- (cu:386-391)
    diff = P.pradius - (pos.z - P.bound_min.z) * ss;
    if (diff > kEpsilon) {
        float3 nrm = make_float3(0.0f, 0.0f, 1.0f);
        adj = P.bound_stiff * diff - P.bound_damp * (nrm.x * veval.x + nrm.y * veval.y + nrm.z * veval.z);
        accel.x += nrm.x * adj; accel.y += nrm.y * adj; accel.z += nrm.z * adj;
    }
    // Z+ (cu:392-397)
    diff = P.pradius - (P.bound_max.z - pos.z) * ss;
    if (diff > kEpsilon) {
        float3 nrm = make_float3(0.0f, 0.0f, -1.0f);
        adj = P.bound_stiff * diff - P.bound_damp * (nrm.x * veval.x + nrm.y * veval.y + nrm.z * veval.z);
        accel.x += nrm.x * adj; accel.y += nrm.y * adj; accel.z += nrm.z * adj;
    }
    accel.x += P.gravity.x; accel.y += P.gravity.y; accel.z += P.gravity.z;
    // accel limit (cu:403-406)
    float speed = accel.x * accel.x + accel.y * accel.y + accel.z * accel.z;
    if (speed > P.AL2) {
        const float k = P.AL / sqrtf(speed);
        accel.x *= k; accel.y *= k; accel.z *= k;
    }
    // velocity limit (cu:409-413)
    speed = vel.x * vel.x + vel.y * vel.y + vel.z * vel.z;
    if (speed > P.VL2) {
        const float k = P.VL / sqrtf(speed);
        vel.x *= k; vel.y *= k; vel.z *= k;
    }
    // leapfrog (cu:416-419)
    const float3 vnext = make_float3(accel.x * dt + vel.x, accel.y * dt + vel.y, accel.z * dt + vel.z);
    veval_o = make_float3((vel.x + vnext.x) * 0.5f, (vel.y + vnext.y) * 0.5f, (vel.z + vnext.z) * 0.5f);
    vel_o = vnext;
    const float dts = dt / ss;
    pos_o = make_float3(pos.x + vnext.x * dts, pos.y + vnext.y * dts, pos.z + vnext.z * dts);
}

// Adjoint (reverse-mode derivative) of the fused SPH step, for sm_103a.
//
// One step maps (x, v, e) -- position, velocity, evaluated velocity in
// pre-sort order -- to the next (x, v, e) in sorted order:
//   sort     X = x[src], V = v[src], E = e[src]                (a permutation)
//   density  rho_s = m poly6 sum_j ((rd2 - |X_s - X_j|^2) d2)^3,  rho = 1 if no pairs
//   force    F_s = sum_j (pterm_sj D + vterm (E_j - E_s)) B_sj,
//            D = X_s - X_j, r = |D| ss, c = h - r, pterm = ss (-1/2) spiky c (p_s + p_j) / r,
//            p = (rho - rho0) kappa, B = c / (rho_s rho_j)
//   advance  a = m F + walls(X, E) + g, clamped to AccelLimit; V clamped to
//            VelLimit; v' = a dt + V; e' = (V + v') / 2; x' = X + v' dt / ss
// (fluids4.0/fluid_kernels.cu: computePressure 112-149, computeForce
// 180-217, advanceParticles 332-420). The integer structure -- cells, the
// permutation, which pairs pass 0 < d^2 < rd2, which walls and limits act --
// is piecewise constant and carries no derivative.
//
// The reverse pass of one step runs on the recomputed forward state of that
// step (sorted X, V, E, rho, F and the grid) in four launches:
//   k_adj_advance   per point: the advance's adjoint; dL/dF, dL/dV (written
//                   through the permutation) and the direct parts of dL/dX, dL/dE
//   k_adj_force     per point s, over its own pairs (s the owner) and its
//                   reverse pairs (the points whose search block holds s):
//                   dL/dX, dL/dE, dL/drho and the parameter partials
//   k_adj_density   per point, own and reverse pairs: the density's share of
//                   dL/dX, written through the permutation
//   k_param_*       deterministic per-scene sums of the parameter partials
// Every sum is a per-thread gather (no atomics), so the result is
// bit-reproducible from run to run. The search block of a point in cell c
// is c-1 .. c+gridSrch-2 per axis, so the points that hold s in their block
// sit in cells c_s-(gridSrch-2) .. c_s+1; the pair test is symmetric in
// FP32 ((a-b) = -(b-a) exactly), so the reverse walk finds exactly the
// transposed pairs.
#include "fl_internal.h"

namespace {

#include "fl_device.cuh"

constexpr int kAdjThreads = 128;
constexpr int kReduceThreads = 256;
constexpr int kReduceChunk = 4096;   // points per partial-sum block

__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 sub3(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 axpy3(float a, float3 x, float3 y) {
    return make_float3(a * x.x + y.x, a * x.y + y.y, a * x.z + y.z);
}

// Acceleration before the AccelLimit clamp: advanceParticles' wall, force
// and gravity terms (fluid_kernels.cu:343-400) in the forward's order.
__device__ __forceinline__ float3 accel_before_clamp(const DevParams &P, float time, float ss, float3 f,
                                                     float3 pos, float3 ve) {
    float3 a = make_float3(f.x * P.pmass, f.y * P.pmass, f.z * P.pmass);
    float diff, adj;
    diff = P.pradius - (pos.y - (P.bound_min.y + (pos.x - P.bound_min.x) * P.bound_slope)) * ss;
    if (diff > kEpsilon) {
        float3 nrm = make_float3(-P.bound_slope, 1.0f - P.bound_slope, 0.0f);
        adj = P.bound_stiff * diff - P.bound_damp * (nrm.x * ve.x + nrm.y * ve.y + nrm.z * ve.z);
        nrm.x *= adj; nrm.y *= adj; nrm.z *= adj;
        a.x += nrm.x - ve.x * P.bound_friction;
        a.y += nrm.y - ve.y * P.bound_friction;
        a.z += nrm.z - ve.z * P.bound_friction;
    }
    diff = P.pradius - (P.bound_max.y - pos.y) * ss;
    if (diff > kEpsilon) {
        float3 nrm = make_float3(0.0f, -1.0f, 0.0f);
        adj = P.bound_stiff * diff - P.bound_damp * (nrm.x * ve.x + nrm.y * ve.y + nrm.z * ve.z);
        nrm.x *= adj; nrm.y *= adj; nrm.z *= adj;
        a.x += nrm.x - ve.x * P.bound_friction;
        a.y += nrm.y - ve.y * P.bound_friction;
        a.z += nrm.z - ve.z * P.bound_friction;
    }
    const float wall = (sinf(time * P.bound_wall_freq + pos.z / 400.f) * 0.5f + 0.5f) * P.bound_wall_force;
    diff = P.pradius - (pos.x - (P.bound_min.x + wall)) * ss;
    if (diff > kEpsilon) a.x += wall * P.bound_stiff * diff - P.bound_damp * ve.x;
    diff = P.pradius - (P.bound_max.x - pos.x) * ss;
    if (diff > kEpsilon) a.x += -(P.bound_stiff * diff - P.bound_damp * (-ve.x));
    diff = P.pradius - (pos.z - P.bound_min.z) * ss;
    if (diff > kEpsilon) a.z += P.bound_stiff * diff - P.bound_damp * ve.z;
    diff = P.pradius - (P.bound_max.z - pos.z) * ss;
    if (diff > kEpsilon) a.z += -(P.bound_stiff * diff - P.bound_damp * (-ve.z));
    a.x += P.gravity.x; a.y += P.gravity.y; a.z += P.gravity.z;
    return a;
}

// Adjoint of the wall terms: given ab = dL/da, adds (da/dX)^T ab to xb and
// (da/dE)^T ab to eb, with each wall active where the forward found it so.
__device__ __forceinline__ void walls_adjoint(const DevParams &P, float time, float ss, float3 pos, float3 ab,
                                              float3 &xb, float3 &eb) {
    float diff;
    diff = P.pradius - (pos.y - (P.bound_min.y + (pos.x - P.bound_min.x) * P.bound_slope)) * ss;
    if (diff > kEpsilon) {
        const float nx = -P.bound_slope, ny = 1.0f - P.bound_slope;
        const float nab = nx * ab.x + ny * ab.y;   // (d a / d adj) . ab
        xb.x += P.bound_stiff * nab * (ss * P.bound_slope);
        xb.y -= P.bound_stiff * nab * ss;
        eb.x += -P.bound_damp * nx * nab - P.bound_friction * ab.x;
        eb.y += -P.bound_damp * ny * nab - P.bound_friction * ab.y;
        eb.z += -P.bound_friction * ab.z;
    }
    diff = P.pradius - (P.bound_max.y - pos.y) * ss;
    if (diff > kEpsilon) {
        const float nab = -ab.y;
        xb.y += P.bound_stiff * nab * ss;
        eb.y += P.bound_damp * nab - P.bound_friction * ab.y;
        eb.x -= P.bound_friction * ab.x;
        eb.z -= P.bound_friction * ab.z;
    }
    const float ph = time * P.bound_wall_freq + pos.z / 400.f;
    const float wall = (sinf(ph) * 0.5f + 0.5f) * P.bound_wall_force;
    diff = P.pradius - (pos.x - (P.bound_min.x + wall)) * ss;
    if (diff > kEpsilon) {
        const float dwall = cosf(ph) * 0.5f * P.bound_wall_force / 400.f;
        xb.x -= ab.x * wall * P.bound_stiff * ss;
        xb.z += ab.x * P.bound_stiff * dwall * (diff + wall * ss);
        eb.x -= P.bound_damp * ab.x;
    }
    diff = P.pradius - (P.bound_max.x - pos.x) * ss;
    if (diff > kEpsilon) {
        xb.x -= ab.x * P.bound_stiff * ss;
        eb.x -= P.bound_damp * ab.x;
    }
    diff = P.pradius - (pos.z - P.bound_min.z) * ss;
    if (diff > kEpsilon) {
        xb.z -= ab.z * P.bound_stiff * ss;
        eb.z -= P.bound_damp * ab.z;
    }
    diff = P.pradius - (P.bound_max.z - pos.z) * ss;
    if (diff > kEpsilon) {
        xb.z -= ab.z * P.bound_stiff * ss;
        eb.z -= P.bound_damp * ab.z;
    }
}

// Adjoint of u -> u L / |u|: (L / |u|) (ub - u (u . ub) / |u|^2).
__device__ __forceinline__ float3 clamp_adjoint(float3 u, float L, float3 ub) {
    const float nn = u.x * u.x + u.y * u.y + u.z * u.z;
    const float k = L / sqrtf(nn);
    const float d = dot3(u, ub) / nn;
    return make_float3(k * (ub.x - u.x * d), k * (ub.y - u.y * d), k * (ub.z - u.z * d));
}

// Reverse of advanceParticles for every sorted slot s. In: the adjoint of
// the step's outputs (slot order). Out: dL/dF (fb), the direct parts of
// dL/dX (xa) and dL/dE (ea), and dL/dV, written through the permutation
// to pre-sort index src[s].
template <bool BATCH>
__global__ void __launch_bounds__(kAdjThreads)
k_adj_advance(const __grid_constant__ DevParams P0, const SceneTab T, int n, const float *time_ptr, float dt,
              const uint32_t *__restrict__ gcell, const uint32_t *__restrict__ src,
              const float4 *__restrict__ X, const float4 *__restrict__ V, const float4 *__restrict__ E,
              const float4 *__restrict__ F,
              const float4 *__restrict__ xo_b, const float4 *__restrict__ vo_b, const float4 *__restrict__ eo_b,
              float4 *__restrict__ xa, float4 *__restrict__ ea, float4 *__restrict__ fb,
              float4 *__restrict__ v_out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const DevParams &P = BATCH ? T.params[T.point_scene[s]] : P0;
    const float3 xb_o = xyz(xo_b[s]), vb_o = xyz(vo_b[s]), eb_o = xyz(eo_b[s]);
    const uint32_t dst = src[s];
    if (gcell[s] == kUndef) {
        // parked at -1000 with zero velocity; the evaluated velocity carries over
        xa[s] = make_float4(0.f, 0.f, 0.f, 0.f);
        ea[s] = f4(eb_o);
        fb[s] = make_float4(0.f, 0.f, 0.f, 0.f);
        v_out[dst] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const float ss = P.sim_scale;
    const float time = *time_ptr;
    const float3 pos = xyz(X[s]), vel = xyz(V[s]), ve = xyz(E[s]);
    const float3 a = accel_before_clamp(P, time, ss, xyz(F[s]), pos, ve);
    const float dts = dt / ss;
    // v' feeds x' (dt/ss), e' (1/2) and v'; V feeds v' and e' (1/2)
    const float3 vt = make_float3(vb_o.x + 0.5f * eb_o.x + dts * xb_o.x, vb_o.y + 0.5f * eb_o.y + dts * xb_o.y,
                                  vb_o.z + 0.5f * eb_o.z + dts * xb_o.z);
    float3 ab = make_float3(dt * vt.x, dt * vt.y, dt * vt.z);
    float3 vb = make_float3(vt.x + 0.5f * eb_o.x, vt.y + 0.5f * eb_o.y, vt.z + 0.5f * eb_o.z);
    if (a.x * a.x + a.y * a.y + a.z * a.z > P.AL2) ab = clamp_adjoint(a, P.AL, ab);
    if (vel.x * vel.x + vel.y * vel.y + vel.z * vel.z > P.VL2) vb = clamp_adjoint(vel, P.VL, vb);
    float3 xb = xb_o, eb = make_float3(0.f, 0.f, 0.f);
    walls_adjoint(P, time, ss, pos, ab, xb, eb);
    xa[s] = f4(xb);
    ea[s] = f4(eb);
    fb[s] = make_float4(P.pmass * ab.x, P.pmass * ab.y, P.pmass * ab.z, 0.f);
    v_out[dst] = f4(vb);
}

// One pair's force adjoint. The owner o's force gets
//   t = (pterm D + vterm dE) B,  D = X_o - X_j,  dE = E_j - E_o,
// and fo = dL/dF_o. Returns dL/dD; the caller adds it to the owner's dL/dX
// and subtracts it from the neighbour's.
struct PairAdj {
    float3 dD;        // dL/dD
    float eB;         // vterm B: dL/dE_j = +eB fo, dL/dE_o = -eB fo
    float rho_common; // B (D.fo) A c kappa / r: dL/drho for both ends (before the B/rho term)
    float SF;         // (pterm D + vterm dE) . fo
    float B;
    float DF, dEF, AcR;   // parameter partials: D.fo, dE.fo, A c / r
};

__device__ __forceinline__ PairAdj pair_adjoint(const DevParams &P, float3 D, float3 dE, float dsq,
                                                float rho_o, float rho_j, float3 fo) {
    PairAdj o;
    const float r = sqrtf(dsq * P.d2);
    const float c = P.psmoothradius - r;
    const float A = P.sim_scale * -0.5f * P.spikykern;
    const float Pp = ((rho_o - P.prest_dens) + (rho_j - P.prest_dens)) * P.pintstiff;
    const float AcR = A * c / r;
    const float pterm = AcR * Pp;
    const float RR = rho_o * rho_j;
    const float B = c / RR;
    const float3 sv = make_float3(pterm * D.x + P.vterm * dE.x, pterm * D.y + P.vterm * dE.y,
                                  pterm * D.z + P.vterm * dE.z);
    const float DF = dot3(D, fo);
    const float SF = dot3(sv, fo);
    // d pterm / dD = -A Pp h d2 / r^3 D;  d B / dD = -(d2 / r) / RR D
    const float r3 = r * r * r;
    const float kD = B * DF * (-A * Pp * P.psmoothradius * P.d2 / r3) + SF * (-(P.d2 / r) / RR);
    o.dD = make_float3(B * pterm * fo.x + kD * D.x, B * pterm * fo.y + kD * D.y, B * pterm * fo.z + kD * D.z);
    o.eB = P.vterm * B;
    o.rho_common = B * DF * AcR * P.pintstiff;
    o.SF = SF;
    o.B = B;
    o.DF = DF;
    o.dEF = dot3(dE, fo);
    o.AcR = AcR;
    return o;
}

// The reverse search block of a point in local cell lc: entry k of the
// y,z,x-ordered block (the forward's adjacency order) as a local cell
// index, or -1 when it leaves [1, gridScanMax] (no points live there).
// With pruning (gridSrch 2) `up` receives the axes along which the entry
// reaches into the upper neighbour cell.
__device__ __forceinline__ int reverse_cell(const DevParams &P, int cx, int cy, int cz, int k, uint32_t &up) {
    const int R = P.gridSrch;
    const int x = k % R, z = (k / R) % R, y = k / (R * R);
    const int sh = R - 2;
    const int ox = cx - sh + x, oy = cy - sh + y, oz = cz - sh + z;
    up = (x == R - 1 ? 1u : 0u) | (y == R - 1 ? 2u : 0u) | (z == R - 1 ? 4u : 0u);
    if (ox < 1 || oy < 1 || oz < 1 || ox > P.gridScanMax.x || oy > P.gridScanMax.y || oz > P.gridScanMax.z)
        return -1;
    return (oy * P.gridRes.z + oz) * P.gridRes.x + ox;
}

__device__ __forceinline__ void local_coords(const DevParams &P, int lc, int &cx, int &cy, int &cz) {
    cx = lc % P.gridRes.x;
    const int t = lc / P.gridRes.x;
    cz = t % P.gridRes.z;
    cy = t / P.gridRes.z;
}

// Reverse of computeForce for point s: its own pairs (from the density
// pass's list, or a walk when the list overflowed) and its reverse pairs.
// Writes the complete dL/dE through the permutation, accumulates dL/dX
// into xa, and stores dL/drho and the parameter partials
// (dL/dvisc, dL/drest_density, dL/dIntStiff) of its own pairs.
template <bool PRUNE, bool BATCH>
__global__ void __launch_bounds__(kAdjThreads)
k_adj_force(const __grid_constant__ DevParams P0, const SceneTab T, int n,
            const float4 *__restrict__ pos, const float4 *__restrict__ veval, const float *__restrict__ rho,
            const uint32_t *__restrict__ gcell, const uint32_t *__restrict__ off, const uint32_t *__restrict__ cnt,
            const uint32_t *__restrict__ upbits, const uint32_t *__restrict__ hitlist,
            const uint32_t *__restrict__ hitcnt, const uint32_t *__restrict__ src,
            const float4 *__restrict__ fb, float4 *__restrict__ xa, const float4 *__restrict__ ea,
            float *__restrict__ rb, float4 *__restrict__ pc, float4 *__restrict__ e_out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const DevParams &P = BATCH ? T.params[T.point_scene[s]] : P0;
    const uint32_t gc = gcell[s];
    const uint32_t dst = src[s];
    if (gc == kUndef) {
        e_out[dst] = ea[s];
        rb[s] = 0.0f;
        pc[s] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const float4 p4 = pos[s];
    const float3 X = xyz(p4), Ev = xyz(veval[s]), fs = xyz(fb[s]);
    const float rs = rho[s];
    const uint32_t my_code = __float_as_uint(p4.w);
    float3 xacc = make_float3(0.f, 0.f, 0.f), eacc = make_float3(0.f, 0.f, 0.f);
    float racc = 0.0f, g_visc = 0.0f, g_rest = 0.0f, g_stiff = 0.0f;

    // own pairs: s is the owner, j its neighbour
    auto own = [&](uint32_t j) {
        const float4 q = pos[j];
        const float3 D = sub3(X, xyz(q));
        const float dsq = D.x * D.x + D.y * D.y + D.z * D.z;
        const float rj = rho[j];
        const float3 dE = sub3(xyz(veval[j]), Ev);
        const PairAdj a = pair_adjoint(P, D, dE, dsq, rs, rj, fs);
        xacc.x += a.dD.x; xacc.y += a.dD.y; xacc.z += a.dD.z;
        eacc.x -= a.eB * fs.x; eacc.y -= a.eB * fs.y; eacc.z -= a.eB * fs.z;
        racc += a.rho_common - a.SF * a.B / rs;
        g_visc += P.lapkern * a.dEF * a.B;
        g_rest += a.B * a.DF * a.AcR * (-2.0f * P.pintstiff);
        g_stiff += a.B * a.DF * a.AcR * ((rs - P.prest_dens) + (rj - P.prest_dens));
    };
    const uint32_t nh = hitcnt[s];
    if (nh <= (uint32_t)P.hcap) {
        for (uint32_t t = 0; t < nh; t++) own(hitlist[list_at(P, s, t)]);
    } else {
        const int base = (int)gc - P.nadj;
        for (int c = 0; c < P.gridAdjCnt; c++) {
            CandIter it;
            cand_begin<PRUNE>(it, P, c, base + P.adj[c], my_code, true, off, cnt, upbits);
            uint32_t j;
            while (cand_next<PRUNE>(it, P, upbits, j)) {
                const float4 q = pos[j];
                const float dx = p4.x - q.x, dy = p4.y - q.y, dz = p4.z - q.z;
                const float dsq = dx * dx + dy * dy + dz * dz;
                if (dsq < P.rd2 && dsq > 0.0f) own(j);
            }
        }
    }

    // reverse pairs: o is the owner, s its neighbour
    int cx, cy, cz;
    local_coords(P, (int)gc - P.cell_base, cx, cy, cz);
    for (int k = 0; k < P.gridAdjCnt; k++) {
        uint32_t up;
        const int lc = reverse_cell(P, cx, cy, cz, k, up);
        if (lc < 0) continue;
        if (PRUNE && (my_code & up) != up) continue;   // too far from those upper faces
        const int cell = P.cell_base + lc;
        const uint32_t o0 = off[cell], o1 = o0 + cnt[cell];
        for (uint32_t o = o0; o < o1; o++) {
            const float4 q = pos[o];
            if (PRUNE && ((__float_as_uint(q.w) >> 3) & up) != up) continue;
            const float3 D = sub3(xyz(q), X);
            const float dsq = D.x * D.x + D.y * D.y + D.z * D.z;
            if (!(dsq < P.rd2 && dsq > 0.0f)) continue;
            const float3 fo = xyz(fb[o]);
            const float3 dE = sub3(Ev, xyz(veval[o]));
            const PairAdj a = pair_adjoint(P, D, dE, dsq, rho[o], rs, fo);
            xacc.x -= a.dD.x; xacc.y -= a.dD.y; xacc.z -= a.dD.z;
            eacc.x += a.eB * fo.x; eacc.y += a.eB * fo.y; eacc.z += a.eB * fo.z;
            racc += a.rho_common - a.SF * a.B / rs;
        }
    }
    const float4 x0 = xa[s], e0 = ea[s];
    xa[s] = make_float4(x0.x + xacc.x, x0.y + xacc.y, x0.z + xacc.z, 0.f);
    e_out[dst] = make_float4(e0.x + eacc.x, e0.y + eacc.y, e0.z + eacc.z, 0.f);
    rb[s] = racc;
    pc[s] = make_float4(g_visc, g_rest, g_stiff, 0.f);
}

// Reverse of computePressure for point s: rho_o = m poly6 sum w^3 with
// w = (rd2 - |D|^2) d2 gives dL/dD = -6 d2 w^2 (m poly6 dL/drho_o) D for
// every pair of owner o. Own and reverse pairs as in k_adj_force; the
// finished dL/dX goes through the permutation.
template <bool PRUNE, bool BATCH>
__global__ void __launch_bounds__(kAdjThreads)
k_adj_density(const __grid_constant__ DevParams P0, const SceneTab T, int n,
              const float4 *__restrict__ pos, const uint32_t *__restrict__ gcell,
              const uint32_t *__restrict__ off, const uint32_t *__restrict__ cnt,
              const uint32_t *__restrict__ upbits, const uint32_t *__restrict__ hitlist,
              const uint32_t *__restrict__ hitcnt, const uint32_t *__restrict__ src,
              const float *__restrict__ rb, const float4 *__restrict__ xa, float4 *__restrict__ x_out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const DevParams &P = BATCH ? T.params[T.point_scene[s]] : P0;
    const uint32_t gc = gcell[s];
    const uint32_t dst = src[s];
    const float4 x0 = xa[s];
    if (gc == kUndef) {
        x_out[dst] = x0;
        return;
    }
    const float4 p4 = pos[s];
    const float3 X = xyz(p4);
    const uint32_t my_code = __float_as_uint(p4.w);
    const float kmp = -6.0f * P.d2 * P.pmass * P.poly6kern;
    const float gs = kmp * rb[s];
    float3 xacc = make_float3(0.f, 0.f, 0.f);
    auto own = [&](uint32_t j) {
        const float3 D = sub3(X, xyz(pos[j]));
        const float dsq = D.x * D.x + D.y * D.y + D.z * D.z;
        const float w = (P.rd2 - dsq) * P.d2;
        const float k = gs * w * w;
        xacc.x += k * D.x; xacc.y += k * D.y; xacc.z += k * D.z;
    };
    const uint32_t nh = hitcnt[s];
    if (gs != 0.0f) {
        if (nh <= (uint32_t)P.hcap) {
            for (uint32_t t = 0; t < nh; t++) own(hitlist[list_at(P, s, t)]);
        } else {
            const int base = (int)gc - P.nadj;
            for (int c = 0; c < P.gridAdjCnt; c++) {
                CandIter it;
                cand_begin<PRUNE>(it, P, c, base + P.adj[c], my_code, true, off, cnt, upbits);
                uint32_t j;
                while (cand_next<PRUNE>(it, P, upbits, j)) {
                    const float4 q = pos[j];
                    const float dx = p4.x - q.x, dy = p4.y - q.y, dz = p4.z - q.z;
                    const float dsq = dx * dx + dy * dy + dz * dz;
                    if (dsq < P.rd2 && dsq > 0.0f) own(j);
                }
            }
        }
    }
    int cx, cy, cz;
    local_coords(P, (int)gc - P.cell_base, cx, cy, cz);
    for (int k = 0; k < P.gridAdjCnt; k++) {
        uint32_t up;
        const int lc = reverse_cell(P, cx, cy, cz, k, up);
        if (lc < 0) continue;
        if (PRUNE && (my_code & up) != up) continue;
        const int cell = P.cell_base + lc;
        const uint32_t o0 = off[cell], o1 = o0 + cnt[cell];
        for (uint32_t o = o0; o < o1; o++) {
            const float4 q = pos[o];
            if (PRUNE && ((__float_as_uint(q.w) >> 3) & up) != up) continue;
            const float3 D = sub3(xyz(q), X);
            const float dsq = D.x * D.x + D.y * D.y + D.z * D.z;
            if (!(dsq < P.rd2 && dsq > 0.0f)) continue;
            const float w = (P.rd2 - dsq) * P.d2;
            const float k2 = kmp * rb[o] * w * w;
            xacc.x -= k2 * D.x; xacc.y -= k2 * D.y; xacc.z -= k2 * D.z;
        }
    }
    x_out[dst] = make_float4(x0.x + xacc.x, x0.y + xacc.y, x0.z + xacc.z, 0.f);
}

// Parameter partials summed per scene in double, in a fixed order: block
// (chunk, scene) sums its chunk, then one thread per scene adds the chunk
// sums in chunk order onto the running totals.
__global__ void __launch_bounds__(kReduceThreads)
k_param_partial(const float4 *__restrict__ pc, const int *__restrict__ sbase, const int *__restrict__ sn,
                int nchunks, double *__restrict__ partial) {
    const int chunk = blockIdx.x, scene = blockIdx.y;
    const int b = sbase[scene], m = sn[scene];
    const int lo = chunk * kReduceChunk;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    for (int k = lo + (int)threadIdx.x; k < lo + kReduceChunk && k < m; k += kReduceThreads) {
        const float4 v = pc[b + k];
        a0 += (double)v.x; a1 += (double)v.y; a2 += (double)v.z;
    }
    for (int d = 16; d > 0; d >>= 1) {
        a0 += __shfl_down_sync(0xffffffffu, a0, d);
        a1 += __shfl_down_sync(0xffffffffu, a1, d);
        a2 += __shfl_down_sync(0xffffffffu, a2, d);
    }
    __shared__ double sm[3][kReduceThreads / 32];
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31u) == 0) { sm[0][w] = a0; sm[1][w] = a1; sm[2][w] = a2; }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int k = 0; k < kReduceThreads / 32; k++) t += sm[threadIdx.x][k];
        partial[((size_t)scene * nchunks + chunk) * 3 + threadIdx.x] = t;
    }
}

__global__ void k_param_final(int nscenes, int nchunks, const double *__restrict__ partial,
                              double *__restrict__ acc) {
    const int scene = blockIdx.x * blockDim.x + threadIdx.x;
    if (scene >= nscenes) return;
    for (int j = 0; j < 3; j++) {
        double t = 0.0;
        for (int c = 0; c < nchunks; c++) t += partial[((size_t)scene * nchunks + c) * 3 + j];
        acc[scene * 3 + j] += t;
    }
}

// Identity tracking across recorded steps: out[s] = in[src[s]] (in null:
// out = src; src null: the identity).
__global__ void k_compose(int n, const uint32_t *__restrict__ src, const uint32_t *__restrict__ in,
                          uint32_t *__restrict__ out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    out[s] = src ? (in ? in[src[s]] : src[s]) : (uint32_t)s;
}

}  // namespace

// ---------------------------------------------------------------------------
// Launch wrappers.

static bool adj_prune(const fl_system *s) { return s->D.prune && s->codes_valid; }

int fl_launch_adj_advance(fl_system *s, const float *time_ptr, const float4 *xo_b, const float4 *vo_b,
                          const float4 *eo_b, float4 *xa, float4 *ea, float4 *fb, float4 *v_out) {
    if (s->n == 0) return FL_OK;
    auto kern = s->batched ? k_adj_advance<true> : k_adj_advance<false>;
    kern<<<blocks_for(s->n, kAdjThreads), kAdjThreads, 0, s->stream>>>(
        s->D, fl_scene_tab(s), s->n, time_ptr, s->P.dt, s->f[F_GCELL].cur<uint32_t>(), s->src,
        s->f[F_POS].cur<float4>(), s->f[F_VEL].cur<float4>(), s->f[F_VEVAL].cur<float4>(),
        s->f[F_FORCE].cur<float4>(), xo_b, vo_b, eo_b, xa, ea, fb, v_out);
    FL_LAUNCH_CHECK("adj_advance");
    return FL_OK;
}

int fl_launch_adj_force(fl_system *s, const float4 *fb, float4 *xa, const float4 *ea, float *rb, float4 *pc,
                        float4 *e_out) {
    if (s->n == 0) return FL_OK;
    const bool pr = adj_prune(s);
    auto kern = s->batched ? (pr ? k_adj_force<true, true> : k_adj_force<false, true>)
                           : (pr ? k_adj_force<true, false> : k_adj_force<false, false>);
    kern<<<blocks_for(s->n, kAdjThreads), kAdjThreads, 0, s->stream>>>(
        s->D, fl_scene_tab(s), s->n, s->f[F_POS].cur<float4>(), s->f[F_VEVAL].cur<float4>(),
        s->f[F_PRESS].cur<float>(), s->f[F_GCELL].cur<uint32_t>(), s->off, s->cnt, s->upbits, s->hitlist,
        s->hitcnt, s->src, fb, xa, ea, rb, pc, e_out);
    FL_LAUNCH_CHECK("adj_force");
    return FL_OK;
}

int fl_launch_adj_density(fl_system *s, const float *rb, const float4 *xa, float4 *x_out) {
    if (s->n == 0) return FL_OK;
    const bool pr = adj_prune(s);
    auto kern = s->batched ? (pr ? k_adj_density<true, true> : k_adj_density<false, true>)
                           : (pr ? k_adj_density<true, false> : k_adj_density<false, false>);
    kern<<<blocks_for(s->n, kAdjThreads), kAdjThreads, 0, s->stream>>>(
        s->D, fl_scene_tab(s), s->n, s->f[F_POS].cur<float4>(), s->f[F_GCELL].cur<uint32_t>(), s->off,
        s->cnt, s->upbits, s->hitlist, s->hitcnt, s->src, rb, xa, x_out);
    FL_LAUNCH_CHECK("adj_density");
    return FL_OK;
}

int fl_param_chunks(int max_scene_points) {
    return max_scene_points <= 0 ? 1 : (max_scene_points + kReduceChunk - 1) / kReduceChunk;
}

int fl_launch_param_reduce(fl_system *s, const float4 *pc, const int *sbase, const int *sn, int nchunks,
                           double *partial, double *acc) {
    if (s->n == 0) return FL_OK;
    dim3 grid((unsigned)nchunks, (unsigned)s->nscenes);
    k_param_partial<<<grid, kReduceThreads, 0, s->stream>>>(pc, sbase, sn, nchunks, partial);
    FL_LAUNCH_CHECK("param_partial");
    k_param_final<<<blocks_for(s->nscenes, 128), 128, 0, s->stream>>>(s->nscenes, nchunks, partial, acc);
    FL_LAUNCH_CHECK("param_final");
    return FL_OK;
}

int fl_launch_compose(fl_system *s, int n, const uint32_t *src, const uint32_t *in, uint32_t *out) {
    if (n == 0) return FL_OK;
    k_compose<<<blocks_for(n, kThreads), kThreads, 0, s->stream>>>(n, src, in, out);
    FL_LAUNCH_CHECK("compose");
    return FL_OK;
}

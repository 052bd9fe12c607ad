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
// step (sorted X, V, E, rho, F and the grid):
//   k_adj_advance   per point: the advance's adjoint; dL/dF, dL/dV (written
//                   through the permutation) and the direct parts of dL/dX, dL/dE
//   k_adj_revwalk   per point s: its reverse pairs outside its own cell (the
//                   points whose search block holds s), recorded in a list
//   k_adj_force     per point s, over its own pairs (s the owner) and its
//                   reverse pairs: dL/dX, dL/dE, dL/drho and the parameter
//                   partials
//   k_adj_density   per point, own and reverse pairs (both from lists): the
//                   density's share of dL/dX, written through the permutation
//   k_adj_crowd_*   the same two for points whose lists overflowed, a block
//                   per point
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

// One kernel instantiation serves single-scene and batched systems (the
// scene table is null for a single scene), so a scene's adjoint is the same
// machine code, and the same bits, alone or in a batch.
__device__ __forceinline__ const DevParams &scene_params(const DevParams &P0, const SceneTab &T, int s) {
    return T.params ? T.params[T.point_scene[s]] : P0;
}
constexpr int kReduceThreads = 256;
constexpr int kReduceChunk = 4096;   // points per partial-sum block

__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

// This file is compiled with FMA contraction on (the adjoint has no
// bit-exact target). The branch decisions it shares with the forward --
// which pairs pass 0 < d^2 < rd2, which walls act, whether the limits
// clamp -- are evaluated with explicitly rounded operations (__fmul_rn,
// __fadd_rn, never contracted) in advanceParticles' order, so they match the
// forward's (compiled without contraction) bit for bit.
__device__ __forceinline__ float dsq_rn(float dx, float dy, float dz) {
    return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// advanceParticles' wall distances (fluid_kernels.cu:356-397).
struct Walls {
    float ylo, yhi, xlo, xhi, zlo, zhi;
    float wall, ph;
};

__device__ __forceinline__ Walls wall_terms(const DevParams &P, float time, float ss, float3 pos) {
    Walls w;
    w.ylo = __fsub_rn(P.pradius, __fmul_rn(__fsub_rn(pos.y, __fadd_rn(P.bound_min.y,
                      __fmul_rn(__fsub_rn(pos.x, P.bound_min.x), P.bound_slope))), ss));
    w.yhi = __fsub_rn(P.pradius, __fmul_rn(__fsub_rn(P.bound_max.y, pos.y), ss));
    w.ph = __fadd_rn(__fmul_rn(time, P.bound_wall_freq), __fdiv_rn(pos.z, 400.f));
    // the forward forms this product in double (the reference's literals)
    w.wall = __double2float_rn(__dmul_rn(__dadd_rn(__dmul_rn((double)sinf(w.ph), 0.5), 0.5),
                                         (double)P.bound_wall_force));
    w.xlo = __fsub_rn(P.pradius, __fmul_rn(__fsub_rn(pos.x, __fadd_rn(P.bound_min.x, w.wall)), ss));
    w.xhi = __fsub_rn(P.pradius, __fmul_rn(__fsub_rn(P.bound_max.x, pos.x), ss));
    w.zlo = __fsub_rn(P.pradius, __fmul_rn(__fsub_rn(pos.z, P.bound_min.z), ss));
    w.zhi = __fsub_rn(P.pradius, __fmul_rn(__fsub_rn(P.bound_max.z, pos.z), ss));
    return w;
}

// Acceleration before the AccelLimit clamp (fluid_kernels.cu:343-400),
// rounded like the forward: force times mass, the wall terms, gravity.
// (Terms the forward multiplies by a zero normal component only add a
// signed zero and are left out; the squared length is unchanged.)
__device__ __forceinline__ float3 accel_before_clamp(const DevParams &P, const Walls &w, float3 f, float3 ve) {
    float3 a = make_float3(__fmul_rn(f.x, P.pmass), __fmul_rn(f.y, P.pmass), __fmul_rn(f.z, P.pmass));
    const float kb = P.bound_stiff, kd = P.bound_damp, fr = P.bound_friction;
    if (w.ylo > kEpsilon) {
        const float nx = -P.bound_slope, ny = __fsub_rn(1.0f, P.bound_slope);
        const float dot = __fadd_rn(__fadd_rn(__fmul_rn(nx, ve.x), __fmul_rn(ny, ve.y)), __fmul_rn(0.0f, ve.z));
        const float adj = __fsub_rn(__fmul_rn(kb, w.ylo), __fmul_rn(kd, dot));
        a.x = __fadd_rn(a.x, __fsub_rn(__fmul_rn(nx, adj), __fmul_rn(ve.x, fr)));
        a.y = __fadd_rn(a.y, __fsub_rn(__fmul_rn(ny, adj), __fmul_rn(ve.y, fr)));
        a.z = __fadd_rn(a.z, __fsub_rn(__fmul_rn(0.0f, adj), __fmul_rn(ve.z, fr)));
    }
    if (w.yhi > kEpsilon) {
        const float adj = __fsub_rn(__fmul_rn(kb, w.yhi), __fmul_rn(kd, -ve.y));
        a.x = __fadd_rn(a.x, __fsub_rn(0.0f, __fmul_rn(ve.x, fr)));
        a.y = __fadd_rn(a.y, __fsub_rn(-adj, __fmul_rn(ve.y, fr)));
        a.z = __fadd_rn(a.z, __fsub_rn(0.0f, __fmul_rn(ve.z, fr)));
    }
    if (w.xlo > kEpsilon)
        a.x = __fadd_rn(a.x, __fsub_rn(__fmul_rn(__fmul_rn(w.wall, kb), w.xlo), __fmul_rn(kd, ve.x)));
    if (w.xhi > kEpsilon) a.x = __fadd_rn(a.x, -__fsub_rn(__fmul_rn(kb, w.xhi), __fmul_rn(kd, -ve.x)));
    if (w.zlo > kEpsilon) a.z = __fadd_rn(a.z, __fsub_rn(__fmul_rn(kb, w.zlo), __fmul_rn(kd, ve.z)));
    if (w.zhi > kEpsilon) a.z = __fadd_rn(a.z, -__fsub_rn(__fmul_rn(kb, w.zhi), __fmul_rn(kd, -ve.z)));
    a.x = __fadd_rn(a.x, P.gravity.x);
    a.y = __fadd_rn(a.y, P.gravity.y);
    a.z = __fadd_rn(a.z, P.gravity.z);
    return a;
}

// Adjoint of the wall terms: given ab = dL/da, adds (da/dX)^T ab to xb and
// (da/dE)^T ab to eb, with each wall active where the forward found it so.
__device__ __forceinline__ void walls_adjoint(const DevParams &P, const Walls &w, float ss, float3 ab,
                                              float3 &xb, float3 &eb) {
    if (w.ylo > kEpsilon) {
        const float nx = -P.bound_slope, ny = 1.0f - P.bound_slope;
        const float nab = nx * ab.x + ny * ab.y;   // (d a / d adj) . ab
        xb.x += P.bound_stiff * nab * (ss * P.bound_slope);
        xb.y -= P.bound_stiff * nab * ss;
        eb.x += -P.bound_damp * nx * nab - P.bound_friction * ab.x;
        eb.y += -P.bound_damp * ny * nab - P.bound_friction * ab.y;
        eb.z += -P.bound_friction * ab.z;
    }
    if (w.yhi > kEpsilon) {
        const float nab = -ab.y;
        xb.y += P.bound_stiff * nab * ss;
        eb.y += P.bound_damp * nab - P.bound_friction * ab.y;
        eb.x -= P.bound_friction * ab.x;
        eb.z -= P.bound_friction * ab.z;
    }
    if (w.xlo > kEpsilon) {
        const float dwall = cosf(w.ph) * 0.5f * P.bound_wall_force / 400.f;
        xb.x -= ab.x * w.wall * P.bound_stiff * ss;
        xb.z += ab.x * P.bound_stiff * dwall * (w.xlo + w.wall * ss);
        eb.x -= P.bound_damp * ab.x;
    }
    if (w.xhi > kEpsilon) {
        xb.x -= ab.x * P.bound_stiff * ss;
        eb.x -= P.bound_damp * ab.x;
    }
    if (w.zlo > kEpsilon) {
        xb.z -= ab.z * P.bound_stiff * ss;
        eb.z -= P.bound_damp * ab.z;
    }
    if (w.zhi > kEpsilon) {
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
__global__ void __launch_bounds__(kAdjThreads)
k_adj_advance(const __grid_constant__ DevParams P0, const SceneTab T, int n, const float *time_ptr, float dt,
              const uint32_t *__restrict__ gcell, const uint32_t *__restrict__ src,
              const float4 *__restrict__ X, const float4 *__restrict__ V, const float4 *__restrict__ E,
              const float4 *__restrict__ F, const float *__restrict__ rho,
              const float4 *__restrict__ xo_b, const float4 *__restrict__ vo_b, const float4 *__restrict__ eo_b,
              float4 *__restrict__ xa, float4 *__restrict__ ea, float4 *__restrict__ fb,
              float4 *__restrict__ v_out, float2 *__restrict__ rr) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const DevParams &P = scene_params(P0, T, s);
    const float3 xb_o = xyz(xo_b[s]), vb_o = xyz(vo_b[s]), eb_o = xyz(eo_b[s]);
    const uint32_t dst = src[s];
    if (gcell[s] == kUndef) {
        // parked at -1000 with zero velocity; the evaluated velocity carries over
        xa[s] = make_float4(0.f, 0.f, 0.f, 0.f);
        ea[s] = f4(eb_o);
        fb[s] = make_float4(0.f, 0.f, 0.f, 0.f);
        v_out[dst] = make_float4(0.f, 0.f, 0.f, 0.f);
        rr[s] = make_float2(0.f, 0.f);
        return;
    }
    const float rho_s = rho[s];
    rr[s] = make_float2(rho_s, 1.0f / rho_s);   // density and its reciprocal for the pair passes
    const float ss = P.sim_scale;
    const float time = *time_ptr;
    const float3 pos = xyz(X[s]), vel = xyz(V[s]), ve = xyz(E[s]);
    const Walls w = wall_terms(P, time, ss, pos);
    const float3 a = accel_before_clamp(P, w, xyz(F[s]), ve);
    const float dts = dt / ss;
    // v' feeds x' (dt/ss), e' (1/2) and v'; V feeds v' and e' (1/2)
    const float3 vt = make_float3(vb_o.x + 0.5f * eb_o.x + dts * xb_o.x, vb_o.y + 0.5f * eb_o.y + dts * xb_o.y,
                                  vb_o.z + 0.5f * eb_o.z + dts * xb_o.z);
    float3 ab = make_float3(dt * vt.x, dt * vt.y, dt * vt.z);
    float3 vb = make_float3(vt.x + 0.5f * eb_o.x, vt.y + 0.5f * eb_o.y, vt.z + 0.5f * eb_o.z);
    if (dsq_rn(a.x, a.y, a.z) > P.AL2) ab = clamp_adjoint(a, P.AL, ab);
    if (dsq_rn(vel.x, vel.y, vel.z) > P.VL2) vb = clamp_adjoint(vel, P.VL, vb);
    float3 xb = xb_o, eb = make_float3(0.f, 0.f, 0.f);
    walls_adjoint(P, w, ss, ab, xb, eb);
    xa[s] = f4(xb);
    ea[s] = f4(eb);
    fb[s] = make_float4(P.pmass * ab.x, P.pmass * ab.y, P.pmass * ab.z, 0.f);
    v_out[dst] = f4(vb);
}

// One pair's force adjoint. The owner o's force gets
//   t = (pterm D + vterm dE) B,  D = X_o - X_j,  dE = E_j - E_o,
// with fo = dL/dF_o:
//   dL/dD      = B pterm fo + (B (D.fo) kP - (sv.fo) kB) D,
//                sv = pterm D + vterm dE, kP = -A Pp h d2 / r^3, kB = d2 / (r rho_o rho_j)
//   dL/dE_j    = +vterm B fo,  dL/dE_o = -vterm B fo
//   dL/drho    = B (D.fo) A c kappa / r - (sv.fo) B / rho   (for either end, its own rho)
// Every term is unchanged when D and dE both change sign, so a pair is
// evaluated in the orientation of the point s the thread owns
// (D = X_s - X_q, dE = E_q - E_s) whichever end owns it; the reverse role
// then enters with the opposite sign. No divisions: r from one reciprocal
// square root, 1/(rho_s rho_q) from per-point reciprocals.
constexpr uint32_t kRevFlag = 0x80000000u;    // entry: a reverse pair only (q owns s)
constexpr uint32_t kBothFlag = 0x40000000u;   // entry: an own pair that is also reverse (same cell)
constexpr uint32_t kSlotMask = 0x3fffffffu;

struct PairGeo {
    float3 D, sv;
    float B, pterm, AcR, kP, kB;
};

__device__ __forceinline__ PairGeo pair_geometry(const DevParams &P, float3 D, float3 dE, float dsq, float rho_s,
                                                 float rho_q, float irr) {
    PairGeo g;
    const float r2 = dsq * P.d2;
    const float ir = rsqrtf(r2);
    const float r = r2 * ir;
    const float c = P.psmoothradius - r;
    const float A = P.sim_scale * -0.5f * P.spikykern;
    const float Pp = ((rho_s - P.prest_dens) + (rho_q - P.prest_dens)) * P.pintstiff;
    g.D = D;
    g.AcR = A * c * ir;
    g.pterm = g.AcR * Pp;
    g.B = c * irr;
    g.sv = make_float3(g.pterm * D.x + P.vterm * dE.x, g.pterm * D.y + P.vterm * dE.y,
                       g.pterm * D.z + P.vterm * dE.z);
    g.kP = -A * Pp * P.psmoothradius * P.d2 * (ir * ir * ir);
    g.kB = P.d2 * ir * irr;
    return g;
}

// Per point: accumulated adjoints of one force-adjoint pass.
struct AdjAcc {
    float3 x, e;
    float r, gv, gr, gk;
};

// The cotangent f of one pair's force, entering s's accumulators with sign
// sg (+1: s owns the pair and f = dL/dF_s; -1: q owns it and f = dL/dF_q).
// Returns f . D for the parameter partials.
__device__ __forceinline__ float apply_cotangent(const DevParams &P, AdjAcc &a, const PairGeo &g, float3 f, float sg,
                                                 float irs) {
    const float DF = dot3(g.D, f);
    const float SF = dot3(g.sv, f);
    const float k = g.B * DF * g.kP - SF * g.kB;
    const float bp = g.B * g.pterm;
    a.x.x += sg * (bp * f.x + k * g.D.x);
    a.x.y += sg * (bp * f.y + k * g.D.y);
    a.x.z += sg * (bp * f.z + k * g.D.z);
    const float ke = sg * P.vterm * g.B;
    a.e.x -= ke * f.x; a.e.y -= ke * f.y; a.e.z -= ke * f.z;
    a.r += sg * (g.B * DF * g.AcR * P.pintstiff - SF * g.B * irs);
    return DF;
}

// One entry of s's pair list (own, reverse, or both).
// The neighbour data one pair's adjoint reads: position, evaluated
// velocity, density and its reciprocal, and (for a pair the neighbour owns)
// the neighbour's force cotangent.
struct PairData {
    float4 qp, qe, fq;
    float2 rq2;
};

__device__ __forceinline__ PairData load_pair(uint32_t entry, const float4 *__restrict__ pos,
                                              const float4 *__restrict__ veval, const float2 *__restrict__ rr,
                                              const float4 *__restrict__ fb) {
    const uint32_t q = entry & kSlotMask;
    PairData d;
    d.qp = pos[q];
    d.qe = veval[q];
    d.rq2 = rr[q];
    d.fq = (entry & (kRevFlag | kBothFlag)) ? fb[q] : make_float4(0.f, 0.f, 0.f, 0.f);
    return d;
}

__device__ __forceinline__ void apply_pair(const DevParams &P, AdjAcc &a, float3 X, float3 Ev, float rs, float3 fs,
                                           float irs, uint32_t entry, const PairData &d) {
    const bool rev_only = (entry & kRevFlag) != 0u;
    const bool both = (entry & kBothFlag) != 0u;
    const float3 D = make_float3(X.x - d.qp.x, X.y - d.qp.y, X.z - d.qp.z);
    const float dsq = D.x * D.x + D.y * D.y + D.z * D.z;
    const float3 dE = make_float3(d.qe.x - Ev.x, d.qe.y - Ev.y, d.qe.z - Ev.z);
    const PairGeo g = pair_geometry(P, D, dE, dsq, rs, d.rq2.x, irs * d.rq2.y);
    const float3 fq = xyz(d.fq);
    const float DF = apply_cotangent(P, a, g, rev_only ? fq : fs, rev_only ? -1.0f : 1.0f, irs);
    if (!rev_only) {
        a.gv += P.lapkern * dot3(dE, fs) * g.B;
        a.gr += g.B * DF * g.AcR * (-2.0f * P.pintstiff);
        a.gk += g.B * DF * g.AcR * ((rs - P.prest_dens) + (d.rq2.x - P.prest_dens));
    }
    if (both) apply_cotangent(P, a, g, fq, -1.0f, irs);
}

__device__ __forceinline__ void adj_pair(const DevParams &P, AdjAcc &a, float3 X, float3 Ev, float rs, float3 fs,
                                         float irs, uint32_t entry, const float4 *__restrict__ pos,
                                         const float4 *__restrict__ veval, const float2 *__restrict__ rr,
                                         const float4 *__restrict__ fb) {
    apply_pair(P, a, X, Ev, rs, fs, irs, entry, load_pair(entry, pos, veval, rr, fb));
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

// Candidates of a point's reverse search block, one at a time in
// ascending cell-entry and slot order, leaving out the point's own cell
// (its pairs there are symmetric: every own pair in the same cell is also a
// reverse pair, taken from the own list instead). With pruning (gridSrch 2)
// a cell that the block reaches into from below along some axes is skipped
// unless the point lies within the band of its upper face on those axes
// (`up`), and only members flagged within the band of their lower face on
// those axes (lower-band rows of the slot flags) are visited, 32 slots per
// flag word.
struct RevIter {
    int k, cx, cy, cz;
    uint32_t gc, code, up;
    uint32_t w, w_last, lo, hi, bits;
};

template <bool PRUNE>
__device__ __forceinline__ uint32_t rev_word(const RevIter &it, const DevParams &P,
                                             const uint32_t *__restrict__ lobits, uint32_t w) {
    uint32_t v = 0xffffffffu;
    if (PRUNE) {
        if (it.up & 1u) v &= lobits[w];
        if (it.up & 2u) v &= lobits[(size_t)P.upwords + w];
        if (it.up & 4u) v &= lobits[2 * (size_t)P.upwords + w];
    }
    if (w == (it.lo >> 5)) v &= 0xffffffffu << (it.lo & 31u);
    if (w == it.w_last && (it.hi & 31u)) v &= 0xffffffffu >> (32u - (it.hi & 31u));
    return v;
}

template <bool PRUNE>
__device__ __forceinline__ void rev_begin(RevIter &it, const DevParams &P, uint32_t gc, uint32_t code, bool active) {
    it.k = active ? 0 : P.gridAdjCnt;
    it.gc = gc;
    it.code = code;
    it.up = 0;
    it.w = it.w_last = it.lo = it.hi = 0;
    it.bits = 0;
    local_coords(P, active ? (int)gc - P.cell_base : 0, it.cx, it.cy, it.cz);
}

// Entry k of the reverse block: false when it leaves the scan range, is the
// own cell, is pruned or is empty; else its slot range and word span.
template <bool PRUNE>
__device__ __forceinline__ bool rev_entry(RevIter &it, const DevParams &P, int k,
                                          const uint32_t *__restrict__ off, const uint32_t *__restrict__ cnt) {
    uint32_t up;
    int cell;
    if (PRUNE) {
        // gridSrch 2: the block is cells c .. c+1 per axis, entry k at offset
        // (k & 1, k >> 2, (k >> 1) & 1) in x, y, z; entry 0 is the own cell
        const int x = k & 1, z = (k >> 1) & 1, y = k >> 2;
        if (k == 0) return false;
        if (it.cx + x > P.gridScanMax.x || it.cy + y > P.gridScanMax.y || it.cz + z > P.gridScanMax.z) return false;
        up = (uint32_t)(x | (y << 1) | (z << 2));
        if ((it.code & up) != up) return false;
        cell = (int)it.gc + x + P.gridRes.x * (z + P.gridRes.z * y);
    } else {
        const int lc = reverse_cell(P, it.cx, it.cy, it.cz, k, up);
        if (lc < 0) return false;
        const int R = P.gridSrch, sh = R - 2;
        if (k % R == sh && (k / R) % R == sh && k / (R * R) == sh) return false;   // own cell
        cell = P.cell_base + lc;
    }
    const uint32_t m = cnt[cell];
    if (m == 0) return false;
    it.up = up;
    it.lo = off[cell];
    it.hi = it.lo + m;
    it.w = it.lo >> 5;
    it.w_last = (it.hi - 1) >> 5;
    return true;
}

template <bool PRUNE>
__device__ __forceinline__ bool rev_next(RevIter &it, const DevParams &P, const uint32_t *__restrict__ off,
                                         const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ lobits,
                                         uint32_t &q) {
    while (it.bits == 0) {
        if (it.w < it.w_last) {
            it.w++;
            it.bits = rev_word<PRUNE>(it, P, lobits, it.w);
            continue;
        }
        // next cell of the reverse block
        bool found = false;
        while (it.k < P.gridAdjCnt) {
            if (rev_entry<PRUNE>(it, P, it.k++, off, cnt)) {
                it.bits = rev_word<PRUNE>(it, P, lobits, it.w);
                found = true;
                break;
            }
        }
        if (!found) return false;
    }
    q = (it.w << 5) + (uint32_t)(__ffs(it.bits) - 1);
    it.bits &= it.bits - 1u;
    return true;
}


// Points whose own or reverse pair list overflowed, appended by k_adj_force
// and walked by the crowd kernels (below).
struct CrowdList {
    uint32_t *pts;
    uint32_t *count;   // listed points (cleared before each reverse step)
    uint32_t cap;
};

// The reverse pairs of point s outside its own cell -- the points q whose
// search block holds s and that pass 0 < d^2 < rd2 -- recorded in revlist
// (up to hcap, in ascending cell-entry and slot order) with their count in
// revcnt, for the force and density adjoints; a count of hcap + 1 means
// the list overflowed (the walk stops there). The block's threads take its
// points grouped by upper-band bits, which decide the cells of the reverse
// block a point visits (all threads of the block call it, with
// grouping_smem(blockDim, kBandKeys) bytes of dynamic shared memory).
template <bool PRUNE>
__device__ __forceinline__ void rev_walk_point(const DevParams &P, int s, const float4 *__restrict__ pos,
                                               const uint32_t *__restrict__ gcell, const uint32_t *__restrict__ off,
                                               const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ upbits,
                                               uint32_t *__restrict__ revlist, uint32_t *__restrict__ revcnt) {
    const uint32_t gc = gcell[s];
    uint32_t nrev = 0;
    if (gc != kUndef) {
        const float4 p4 = pos[s];
        const uint32_t hcap = (uint32_t)P.hcap;
        const uint32_t *lobits = upbits + 3 * (size_t)P.upwords;
        RevIter it;
        rev_begin<PRUNE>(it, P, gc, __float_as_uint(p4.w), true);
        // one cell of the reverse block at a time (the lanes of a warp meet at
        // each cell's end), 32 slots per flag word, ascending
        for (int k = 0; k < P.gridAdjCnt && nrev <= hcap; k++) {
            if (!rev_entry<PRUNE>(it, P, k, off, cnt)) continue;
            for (uint32_t w = it.lo >> 5; w <= it.w_last && nrev <= hcap; w++) {
                uint32_t bits = rev_word<PRUNE>(it, P, lobits, w);
                while (bits) {
                    const uint32_t q = (w << 5) + (uint32_t)(__ffs(bits) - 1);
                    bits &= bits - 1u;
                    const float4 qp = pos[q];
                    const float dsq = dsq_rn(qp.x - p4.x, qp.y - p4.y, qp.z - p4.z);
                    if (dsq < P.rd2 && dsq > 0.0f) {
                        if (nrev == hcap) { nrev++; break; }   // overflowed: the consumers walk again
                        revlist[list_at(P, s, nrev)] = q;
                        nrev++;
                    }
                }
            }
        }
    }
    revcnt[s] = nrev;
}

template <bool PRUNE>
__global__ void __launch_bounds__(kThreads)
k_adj_revwalk(const __grid_constant__ DevParams P0, const SceneTab T, int n, const float4 *__restrict__ pos,
              const uint32_t *__restrict__ gcell, const uint32_t *__restrict__ off,
              const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ upbits,
              uint32_t *__restrict__ revlist, uint32_t *__restrict__ revcnt) {
    extern __shared__ uint32_t s_dyn[];
    const int s = PRUNE ? band_grouped_slot(n, pos, gcell, 0, s_dyn) : (int)(blockIdx.x * blockDim.x + threadIdx.x);
    if (s >= n) return;
    rev_walk_point<PRUNE>(scene_params(P0, T, s), s, pos, gcell, off, cnt, upbits, revlist, revcnt);
}

// The walk for the points k_adj_revsort listed (reverse lists too long to
// sort in registers), a grid-stride loop over the listed count.
template <bool PRUNE>
__global__ void __launch_bounds__(kThreads)
k_adj_revwalk_listed(const __grid_constant__ DevParams P0, const SceneTab T, const float4 *__restrict__ pos,
                     const uint32_t *__restrict__ gcell, const uint32_t *__restrict__ off,
                     const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ upbits,
                     const uint32_t *__restrict__ listed, const uint32_t *__restrict__ listed_count,
                     uint32_t *__restrict__ revlist, uint32_t *__restrict__ revcnt) {
    const uint32_t m = *listed_count;
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
        const int s = (int)listed[k];
        rev_walk_point<PRUNE>(scene_params(P0, T, s), s, pos, gcell, off, cnt, upbits, revlist, revcnt);
    }
}

// The same reverse lists by transposing the density pass's pair lists
// (one thread per owner q; the walk above is kept for comparison): every
// pair (q, s) of q's list with s outside q's cell is a reverse pair of s
// outside its own cell, and the pair lists hold exactly the pairs that pass
// (the test is symmetric). Each is appended to s's list at a position taken
// from s's count by an atomic; k_adj_revsort then puts every list in
// ascending slot order, the walk's order (the reverse block's cells in
// ascending index, each in ascending slot), so consumers see the same
// lists. An owner whose own list overflowed walks its search block again.
// revcnt must be zero before the launch.
constexpr uint32_t kScatterBatch = 4;

template <bool PRUNE>
__global__ void __launch_bounds__(kThreads)
k_adj_revscatter(const __grid_constant__ DevParams P0, const SceneTab T, int n, const float4 *__restrict__ pos,
                 const uint32_t *__restrict__ gcell, const uint32_t *__restrict__ off,
                 const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ upbits,
                 const uint32_t *__restrict__ hitlist, const uint32_t *__restrict__ hitcnt,
                 uint32_t *__restrict__ revlist, uint32_t *__restrict__ revcnt) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const uint32_t gq = gcell[q];
    if (gq == kUndef) return;
    const DevParams &P = scene_params(P0, T, q);
    const uint32_t hcap = (uint32_t)P.hcap;
    auto push = [&](uint32_t s) {
        if (gcell[s] == gq) return;   // in q's cell: a pair of s's own cell
        const uint32_t at = atomicAdd(&revcnt[s], 1u);
        if (at < hcap) revlist[list_at(P, (int)s, at)] = (uint32_t)q;
    };
    const uint32_t nh = hitcnt[q];
    if (nh <= hcap) {
        // four entries per round: their list words, cells and count atomics
        // are each requested before the first is waited for
        for (uint32_t t = 0; t < nh; t += kScatterBatch) {
            uint32_t sj[kScatterBatch], at[kScatterBatch];
#pragma unroll
            for (uint32_t k = 0; k < kScatterBatch; k++)
                sj[k] = (t + k < nh) ? hitlist[list_at(P, q, t + k)] : kUndef;
#pragma unroll
            for (uint32_t k = 0; k < kScatterBatch; k++)
                at[k] = (sj[k] != kUndef && gcell[sj[k]] != gq) ? 0u : hcap;
#pragma unroll
            for (uint32_t k = 0; k < kScatterBatch; k++)
                if (at[k] == 0u) at[k] = atomicAdd(&revcnt[sj[k]], 1u);
#pragma unroll
            for (uint32_t k = 0; k < kScatterBatch; k++)
                if (at[k] < hcap) revlist[list_at(P, (int)sj[k], at[k])] = (uint32_t)q;
        }
        return;
    }
    const float4 p = pos[q];
    const int base = (int)gq - P.nadj;
    for (int c = 0; c < P.gridAdjCnt; c++) {
        CandIter it;
        cand_begin<PRUNE>(it, P, c, base + P.adj[c], __float_as_uint(p.w), true, off, cnt, upbits);
        uint32_t j;
        while (cand_next<PRUNE>(it, P, upbits, j)) {
            const float4 o = pos[j];
            const float dsq = dsq_rn(p.x - o.x, p.y - o.y, p.z - o.z);
            if (dsq < P.rd2 && dsq > 0.0f) push(j);
        }
    }
}

// Ascending order for each reverse list of k_adj_revscatter: up to 32
// entries by a bitonic network in registers (a warp runs the network its
// longest list needs); a longer list is listed for k_adj_revwalk_listed,
// which writes it again by walking; a count above hcap becomes hcap + 1,
// the walk's overflow mark.
template <int N>
__device__ __forceinline__ void sort_row(uint32_t *row, uint32_t c) {   // entry t at row[32 t]
    uint32_t r[N];
#pragma unroll
    for (int t = 0; t < N; t++) r[t] = ((uint32_t)t < c) ? row[32 * t] : 0xffffffffu;
#pragma unroll
    for (int k = 2; k <= N; k <<= 1)
#pragma unroll
        for (int j = k >> 1; j > 0; j >>= 1)
#pragma unroll
            for (int i = 0; i < N; i++) {
                const int l = i ^ j;
                if (l > i) {
                    const uint32_t lo = min(r[i], r[l]), hi = max(r[i], r[l]);
                    const bool up = (i & k) == 0;
                    r[i] = up ? lo : hi;
                    r[l] = up ? hi : lo;
                }
            }
#pragma unroll
    for (int t = 0; t < N; t++)
        if ((uint32_t)t < c) row[32 * t] = r[t];
}

__global__ void __launch_bounds__(kThreads)
k_adj_revsort(int n, int hcap_in, uint32_t *__restrict__ revlist, uint32_t *__restrict__ revcnt,
              uint32_t *__restrict__ listed, uint32_t *__restrict__ listed_count) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (blockIdx.x * blockDim.x + (threadIdx.x & ~31u) >= (unsigned)n) return;   // whole warp past n
    const uint32_t hcap = (uint32_t)hcap_in;
    uint32_t c = (s < n) ? revcnt[s] : 0u;
    if (c > hcap) {
        revcnt[s] = hcap + 1;
        c = 0;
    } else if (c > 32) {
        listed[atomicAdd(listed_count, 1u)] = (uint32_t)s;
        c = 0;
    }
    if (c < 2) c = 0;
    // one network per warp, the size its longest list needs
    const uint32_t most = __reduce_max_sync(0xffffffffu, c);
    if (most == 0) return;
    uint32_t *row = revlist + ((size_t)(s >> 5) * hcap) * 32u + (uint32_t)(s & 31);
    if (most <= 8) sort_row<8>(row, c);
    else if (most <= 16) sort_row<16>(row, c);
    else sort_row<32>(row, c);
}

// Reverse of computeForce for point s (all 32 lanes of a warp call it):
// the warp evaluates, in step, every lane's own pairs (the density pass's
// list; those in the own cell are reverse pairs too) and its reverse pairs
// (k_adj_revwalk's list), so the long pair arithmetic runs with the lanes
// busy. A point whose own or reverse list overflowed is appended to the
// crowd list instead, and k_adj_crowd_force adds those pairs. Writes dL/dE
// through the permutation, accumulates dL/dX into xa, stores dL/drho and
// the parameter partials (dL/dvisc, dL/drest_density, dL/dIntStiff) of its
// own pairs.
template <bool PRUNE>
__global__ void __launch_bounds__(kAdjThreads, 8)
k_adj_force(const __grid_constant__ DevParams P0, const SceneTab T, int n,
            const float4 *__restrict__ pos, const float4 *__restrict__ veval, const float2 *__restrict__ rr,
            const uint32_t *__restrict__ gcell, const uint32_t *__restrict__ off, const uint32_t *__restrict__ cnt,
            const uint32_t *__restrict__ upbits, const uint32_t *__restrict__ hitlist,
            const uint32_t *__restrict__ hitcnt, const uint32_t *__restrict__ src,
            const float4 *__restrict__ fb, float4 *__restrict__ xa, const float4 *__restrict__ ea,
            float *__restrict__ rb, float4 *__restrict__ pc, float4 *__restrict__ e_out,
            const uint32_t *__restrict__ revlist, const uint32_t *__restrict__ revcnt, const CrowdList crowd) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    const DevParams &P = scene_params(P0, T, s < n ? s : 0);
    const uint32_t gc = (s < n) ? gcell[s] : kUndef;
    const bool active = gc != kUndef;
    AdjAcc acc;
    acc.x = acc.e = make_float3(0.f, 0.f, 0.f);
    acc.r = acc.gv = acc.gr = acc.gk = 0.0f;
    float3 X = make_float3(0.f, 0.f, 0.f), Ev = X, fs = X;
    float rs = 1.0f, irs = 1.0f;
    uint32_t my_code = 0, c_lo = 0, c_hi = 0;
    if (active) {
        const float4 p4 = pos[s];
        X = xyz(p4);
        my_code = __float_as_uint(p4.w);
        Ev = xyz(veval[s]);
        fs = xyz(fb[s]);
        const float2 r2 = rr[s];
        rs = r2.x;
        irs = r2.y;
        c_lo = off[gc];
        c_hi = c_lo + cnt[gc];
    }
    const uint32_t hcap = (uint32_t)P.hcap;
    const uint32_t *lobits = upbits + 3 * (size_t)P.upwords;
    const uint32_t nrev = active ? revcnt[s] : 0u;

    // own pairs (own cell: both roles) and reverse pairs from the lists
    auto own_entry = [&](uint32_t j) { return (j >= c_lo && j < c_hi) ? (j | kBothFlag) : j; };
    const uint32_t nh = active ? hitcnt[s] : 0u;
    const uint32_t n_own = (nh <= hcap) ? nh : 0u;
    const uint32_t n_rev = (nrev <= hcap) ? nrev : 0u;
    const uint32_t mine = n_own + n_rev;
    const uint32_t most = __reduce_max_sync(0xffffffffu, mine);
    for (uint32_t t = 0; t < most; t++) {
        if (t < mine) {
            const uint32_t e = (t < n_own) ? own_entry(hitlist[list_at(P, s, t)])
                                           : (revlist[list_at(P, s, t - n_own)] | kRevFlag);
            adj_pair(P, acc, X, Ev, rs, fs, irs, e, pos, veval, rr, fb);
        }
    }

    // overflowed lists: the point's walks go to the crowd kernels
    if (active && (nh > hcap || nrev > hcap)) {
        const uint32_t slot = atomicAdd(crowd.count, 1u);
        if (slot < crowd.cap) crowd.pts[slot] = (uint32_t)s;
    }

    if (s >= n) return;
    const uint32_t dst = src[s];
    if (!active) {
        e_out[dst] = ea[s];
        rb[s] = 0.0f;
        pc[s] = make_float4(0.f, 0.f, 0.f, 0.f);
        return;
    }
    const float4 x0 = xa[s], e0 = ea[s];
    xa[s] = make_float4(x0.x + acc.x.x, x0.y + acc.x.y, x0.z + acc.x.z, 0.f);
    e_out[dst] = make_float4(e0.x + acc.e.x, e0.y + acc.e.y, e0.z + acc.e.z, 0.f);
    rb[s] = acc.r;
    pc[s] = make_float4(acc.gv, acc.gr, acc.gk, 0.f);
}

// Reverse of computePressure for point s: rho_o = m poly6 sum w^3 with
// w = (rd2 - |D|^2) d2 gives dL/dD = -6 d2 w^2 (m poly6 dL/drho_o) D for
// every pair of owner o. Own pairs from the density pass's list (those in
// the point's own cell are reverse pairs too), reverse pairs in the other
// cells from the list k_adj_revwalk recorded; the finished dL/dX goes
// through the permutation. With walk_overflow off (as fl_backward launches
// it) a point whose list overflowed is left to k_adj_crowd_density, which
// spreads its pairs over a block; on, the point walks them itself. (The
// per-thread walk is kept compiled in: without it this kernel's list loops
// were given fewer registers and more resident warps, and ran 40% slower
// on the wave tank.)
template <bool PRUNE>
__global__ void __launch_bounds__(kAdjThreads)
k_adj_density(const __grid_constant__ DevParams P0, const SceneTab T, int n,
              const float4 *__restrict__ pos, const uint32_t *__restrict__ gcell,
              const uint32_t *__restrict__ off, const uint32_t *__restrict__ cnt,
              const uint32_t *__restrict__ upbits, const uint32_t *__restrict__ hitlist,
              const uint32_t *__restrict__ hitcnt, const uint32_t *__restrict__ revlist,
              const uint32_t *__restrict__ revcnt, const uint32_t *__restrict__ src,
              const float *__restrict__ rb, const float4 *__restrict__ xa, float4 *__restrict__ x_out,
              bool walk_overflow) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    const DevParams &P = scene_params(P0, T, s);
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
    // own pair (owner s): + gs w^2 (X_s - X_j)
    auto own = [&](uint32_t j) {
        const float4 q = pos[j];
        const float3 D = make_float3(X.x - q.x, X.y - q.y, X.z - q.z);
        const float w = (P.rd2 - (D.x * D.x + D.y * D.y + D.z * D.z)) * P.d2;
        const float k = gs * w * w;
        xacc.x += k * D.x; xacc.y += k * D.y; xacc.z += k * D.z;
    };
    // reverse pair (owner o): - g_o w^2 (X_o - X_s)
    auto rev = [&](uint32_t o) {
        const float4 q = pos[o];
        const float3 D = make_float3(q.x - X.x, q.y - X.y, q.z - X.z);
        const float w = (P.rd2 - (D.x * D.x + D.y * D.y + D.z * D.z)) * P.d2;
        const float k = kmp * rb[o] * w * w;
        xacc.x -= k * D.x; xacc.y -= k * D.y; xacc.z -= k * D.z;
    };
    // own pairs; those in the own cell are reverse pairs as well
    const uint32_t c_lo = off[gc], c_hi = c_lo + cnt[gc];
    auto both = [&](uint32_t j) {
        if (gs != 0.0f) own(j);
        if (j >= c_lo && j < c_hi) rev(j);
    };
    const uint32_t nh = hitcnt[s];
    // the lists are read four entries per round, all requested before the
    // first is used (the pairs still add in list order)
    if (nh <= (uint32_t)P.hcap) {
        uint32_t t = 0;
        for (; t + 4 <= nh; t += 4) {
            uint32_t j[4];
#pragma unroll
            for (int k = 0; k < 4; k++) j[k] = hitlist[list_at(P, s, t + k)];
#pragma unroll
            for (int k = 0; k < 4; k++) both(j[k]);
        }
        for (; t < nh; t++) both(hitlist[list_at(P, s, t)]);
    } else if (walk_overflow) {
        const int base = (int)gc - P.nadj;
        for (int c = 0; c < P.gridAdjCnt; c++) {
            CandIter it;
            cand_begin<PRUNE>(it, P, c, base + P.adj[c], my_code, true, off, cnt, upbits);
            uint32_t j;
            while (cand_next<PRUNE>(it, P, upbits, j)) {
                const float4 q = pos[j];
                const float dsq = dsq_rn(p4.x - q.x, p4.y - q.y, p4.z - q.z);
                if (dsq < P.rd2 && dsq > 0.0f) both(j);
            }
        }
    }
    // reverse pairs in the other cells: the force adjoint's list, or a walk
    const uint32_t nr = revcnt[s];
    if (nr <= (uint32_t)P.hcap) {
        uint32_t t = 0;
        for (; t + 4 <= nr; t += 4) {
            uint32_t o[4];
#pragma unroll
            for (int k = 0; k < 4; k++) o[k] = revlist[list_at(P, s, t + k)];
#pragma unroll
            for (int k = 0; k < 4; k++) rev(o[k]);
        }
        for (; t < nr; t++) rev(revlist[list_at(P, s, t)]);
    } else if (walk_overflow) {
        const uint32_t *lobits = upbits + 3 * (size_t)P.upwords;
        RevIter it;
        rev_begin<PRUNE>(it, P, gc, my_code, true);
        uint32_t o;
        while (rev_next<PRUNE>(it, P, off, cnt, lobits, o)) {
            const float4 q = pos[o];
            const float dsq = dsq_rn(q.x - X.x, q.y - X.y, q.z - X.z);
            if (dsq < P.rd2 && dsq > 0.0f) rev(o);
        }
    }
    x_out[dst] = make_float4(x0.x + xacc.x, x0.y + xacc.y, x0.z + xacc.z, 0.f);
}

// ---------------------------------------------------------------------------
// Crowded points. A point whose own or reverse pair list overflowed (a
// collapsing scene crowds hundreds or thousands of points into a cell) is
// left out of k_adj_force's and k_adj_density's list drains and appended to
// the crowd list; k_adj_crowd_force and k_adj_crowd_density then give each
// listed point a whole block, so its pairs spread over the GPU instead of
// one thread walking them all. The candidates of each walked cell are cut
// into 32-slot chunks counted from the cell's first slot; chunk g of the
// point's walk goes to warp g % warps and lane l of that warp takes slot
// l of the chunk when the band flags keep it. The lanes' sums are added in
// a fixed order, so a point's result is reproducible, and the same alone or
// in a batch (chunks do not depend on where a scene's slots start).
constexpr int kCrowdThreads = 256;

template <bool PRUNE, class F>
__device__ __forceinline__ void crowd_chunks(const DevParams &P, uint32_t gc, uint32_t code, bool own, bool rev,
                                             const uint32_t *__restrict__ off, const uint32_t *__restrict__ cnt,
                                             const uint32_t *__restrict__ upbits, F &&f) {
    const uint32_t lane = lane_id(), warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    uint32_t g = 0;   // chunks of the walk so far (the same on every thread)
    auto cell = [&](uint32_t lo, uint32_t hi, uint32_t axes, const uint32_t *rows, bool is_rev) {
        const uint32_t nq = (hi - lo + 31) >> 5;
        for (uint32_t q = (warp + nwarps - g % nwarps) % nwarps; q < nq; q += nwarps) {
            const uint32_t j = lo + 32 * q + lane;
            if (j >= hi) continue;
            bool keep = true;
            if (PRUNE && axes) {
                const uint32_t w = j >> 5, b = 1u << (j & 31u);
                if ((axes & 1u) && !(rows[w] & b)) keep = false;
                if ((axes & 2u) && !(rows[(size_t)P.upwords + w] & b)) keep = false;
                if ((axes & 4u) && !(rows[2 * (size_t)P.upwords + w] & b)) keep = false;
            }
            if (keep) f(j, is_rev);
        }
        g += nq;
    };
    if (own) {   // the search block, as cand_begin / cand_word prune it
        const int base = (int)gc - P.nadj;
        for (int c = 0; c < P.gridAdjCnt; c++) {
            CandIter it;
            cand_begin<PRUNE>(it, P, c, base + P.adj[c], code, true, off, cnt, upbits);
            if (it.lo < it.hi) cell(it.lo, it.hi, it.U, upbits, false);
        }
    }
    if (rev) {   // the reverse block outside the own cell, as rev_entry / rev_word prune it
        RevIter it;
        rev_begin<PRUNE>(it, P, gc, code, true);
        for (int k = 0; k < P.gridAdjCnt; k++)
            if (rev_entry<PRUNE>(it, P, k, off, cnt)) cell(it.lo, it.hi, it.up, upbits + 3 * (size_t)P.upwords, true);
    }
}

// Sums v[0..K) over the block into s_red (thread 0 reads the totals): each
// warp by a fixed shuffle tree, then the warps in order.
template <int K>
__device__ __forceinline__ void block_sum(float (&v)[K], float (*s_red)[K]) {
#pragma unroll
    for (int k = 0; k < K; k++)
#pragma unroll
        for (int d = 16; d > 0; d >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], d);
    if (lane_id() == 0)
#pragma unroll
        for (int k = 0; k < K; k++) s_red[threadIdx.x >> 5][k] = v[k];
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < K; k++) {
            float t = s_red[0][k];
            for (uint32_t w = 1; w < (blockDim.x >> 5); w++) t += s_red[w][k];
            v[k] = t;
        }
    }
}

// The force adjoint's walked pairs of each crowded point, added to what
// k_adj_force wrote for it (dL/dX, dL/dE through the permutation, dL/drho,
// the parameter partials).
template <bool PRUNE>
__global__ void __launch_bounds__(kCrowdThreads)
k_adj_crowd_force(const __grid_constant__ DevParams P0, const SceneTab T, const float4 *__restrict__ pos,
                  const float4 *__restrict__ veval, const float2 *__restrict__ rr,
                  const uint32_t *__restrict__ gcell, const uint32_t *__restrict__ off,
                  const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ upbits,
                  const uint32_t *__restrict__ hitcnt, const uint32_t *__restrict__ revcnt,
                  const uint32_t *__restrict__ src, const float4 *__restrict__ fb, float4 *__restrict__ xa,
                  float4 *__restrict__ e_out, float *__restrict__ rb, float4 *__restrict__ pc, const CrowdList L) {
    __shared__ float s_red[kCrowdThreads / 32][10];
    __shared__ uint32_t s_nlist;
    if (threadIdx.x == 0) s_nlist = min(*(volatile uint32_t *)L.count, L.cap);
    __syncthreads();
    const uint32_t nlist = s_nlist;
    for (uint32_t b = blockIdx.x; b < nlist; b += gridDim.x) {
        const int s = (int)L.pts[b];
        const DevParams &P = scene_params(P0, T, s);
        const uint32_t gc = gcell[s];
        const float4 p4 = pos[s];
        const float3 X = xyz(p4), Ev = xyz(veval[s]), fs = xyz(fb[s]);
        const float2 r2 = rr[s];
        const uint32_t c_lo = off[gc], c_hi = c_lo + cnt[gc], hcap = (uint32_t)P.hcap;
        AdjAcc part;
        part.x = part.e = make_float3(0.f, 0.f, 0.f);
        part.r = part.gv = part.gr = part.gk = 0.0f;
        crowd_chunks<PRUNE>(P, gc, __float_as_uint(p4.w), hitcnt[s] > hcap, revcnt[s] > hcap, off, cnt, upbits,
                            [&](uint32_t j, bool is_rev) {
            const float4 q = pos[j];
            if (!is_rev) {
                const float dsq = dsq_rn(X.x - q.x, X.y - q.y, X.z - q.z);
                if (dsq < P.rd2 && dsq > 0.0f)
                    adj_pair(P, part, X, Ev, r2.x, fs, r2.y, (j >= c_lo && j < c_hi) ? (j | kBothFlag) : j, pos,
                             veval, rr, fb);
            } else {
                const float dsq = dsq_rn(q.x - X.x, q.y - X.y, q.z - X.z);
                if (dsq < P.rd2 && dsq > 0.0f) adj_pair(P, part, X, Ev, r2.x, fs, r2.y, j | kRevFlag, pos, veval, rr, fb);
            }
        });
        float v[10] = {part.x.x, part.x.y, part.x.z, part.e.x, part.e.y, part.e.z, part.r, part.gv, part.gr, part.gk};
        block_sum<10>(v, s_red);
        if (threadIdx.x == 0) {
            const uint32_t dst = src[s];
            const float4 x0 = xa[s], e0 = e_out[dst], c0 = pc[s];
            xa[s] = make_float4(x0.x + v[0], x0.y + v[1], x0.z + v[2], 0.f);
            e_out[dst] = make_float4(e0.x + v[3], e0.y + v[4], e0.z + v[5], 0.f);
            rb[s] += v[6];
            pc[s] = make_float4(c0.x + v[7], c0.y + v[8], c0.z + v[9], 0.f);
        }
        __syncthreads();
    }
}

// The density adjoint's walked pairs of each crowded point (k_adj_density
// leaves them out when walk_overflow is off), added to the dL/dX
// k_adj_density wrote for it.
template <bool PRUNE>
__global__ void __launch_bounds__(kCrowdThreads)
k_adj_crowd_density(const __grid_constant__ DevParams P0, const SceneTab T, const float4 *__restrict__ pos,
                    const uint32_t *__restrict__ gcell, const uint32_t *__restrict__ off,
                    const uint32_t *__restrict__ cnt, const uint32_t *__restrict__ upbits,
                    const uint32_t *__restrict__ hitcnt, const uint32_t *__restrict__ revcnt,
                    const uint32_t *__restrict__ src, const float *__restrict__ rb, float4 *__restrict__ x_out,
                    const CrowdList L) {
    __shared__ float s_red[kCrowdThreads / 32][3];
    __shared__ uint32_t s_nlist;
    if (threadIdx.x == 0) s_nlist = min(*(volatile uint32_t *)L.count, L.cap);
    __syncthreads();
    const uint32_t nlist = s_nlist;
    for (uint32_t b = blockIdx.x; b < nlist; b += gridDim.x) {
        const int s = (int)L.pts[b];
        const DevParams &P = scene_params(P0, T, s);
        const uint32_t gc = gcell[s];
        const float4 p4 = pos[s];
        const float3 X = xyz(p4);
        const float kmp = -6.0f * P.d2 * P.pmass * P.poly6kern;
        const float gs = kmp * rb[s];
        const uint32_t c_lo = off[gc], c_hi = c_lo + cnt[gc], hcap = (uint32_t)P.hcap;
        float3 part = make_float3(0.f, 0.f, 0.f);
        auto rev = [&](uint32_t o, float4 q) {   // owner o: - g_o w^2 (X_o - X_s)
            const float3 D = make_float3(q.x - X.x, q.y - X.y, q.z - X.z);
            const float w = (P.rd2 - (D.x * D.x + D.y * D.y + D.z * D.z)) * P.d2;
            const float k = kmp * rb[o] * w * w;
            part.x -= k * D.x; part.y -= k * D.y; part.z -= k * D.z;
        };
        crowd_chunks<PRUNE>(P, gc, __float_as_uint(p4.w), hitcnt[s] > hcap, revcnt[s] > hcap, off, cnt, upbits,
                            [&](uint32_t j, bool is_rev) {
            const float4 q = pos[j];
            if (!is_rev) {
                const float dsq = dsq_rn(p4.x - q.x, p4.y - q.y, p4.z - q.z);
                if (dsq < P.rd2 && dsq > 0.0f) {
                    if (gs != 0.0f) {   // owner s: + gs w^2 (X_s - X_j)
                        const float3 D = make_float3(X.x - q.x, X.y - q.y, X.z - q.z);
                        const float w = (P.rd2 - (D.x * D.x + D.y * D.y + D.z * D.z)) * P.d2;
                        const float k = gs * w * w;
                        part.x += k * D.x; part.y += k * D.y; part.z += k * D.z;
                    }
                    if (j >= c_lo && j < c_hi) rev(j, q);
                }
            } else {
                const float dsq = dsq_rn(q.x - X.x, q.y - X.y, q.z - X.z);
                if (dsq < P.rd2 && dsq > 0.0f) rev(j, q);
            }
        });
        float v[3] = {part.x, part.y, part.z};
        block_sum<3>(v, s_red);
        if (threadIdx.x == 0) {
            const uint32_t dst = src[s];
            const float4 x0 = x_out[dst];
            x_out[dst] = make_float4(x0.x + v[0], x0.y + v[1], x0.z + v[2], 0.f);
        }
        __syncthreads();
    }
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
                              const int *__restrict__ gexp, double *__restrict__ acc) {
    // one warp per scene: lane l takes chunks l, l+32, ...; fixed shuffle tree
    const int scene = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (scene >= nscenes) return;
    const unsigned lane = threadIdx.x & 31u;
    for (int j = 0; j < 3; j++) {
        double t = 0.0;
        for (int c = (int)lane; c < nchunks; c += 32) t += partial[((size_t)scene * nchunks + c) * 3 + j];
        for (int d = 16; d > 0; d >>= 1) t += __shfl_xor_sync(0xffffffffu, t, d);
        // the partials carry the cotangent's current scale 2^-gexp
        if (lane == 0) acc[scene * 3 + j] += gexp ? ldexp(t, gexp[scene]) : t;
    }
}

// ---- cotangent renormalisation ----------------------------------------------
// The exact gradient of a long rollout grows about 1.4x per step (nearby
// trajectories diverge), so over a few hundred steps the cotangents leave
// the FP32 range. After each reverse step the cotangents of a scene whose
// largest component exceeds 2^40 are scaled by 2^-k (k its binary
// exponent) and k is added to the scene's exponent. Power-of-two scaling
// is exact and every reverse operation is linear in the cotangent, so the
// mantissas round exactly as the unscaled values would.
constexpr float kRescaleAbove = 1099511627776.0f;   // 2^40

__device__ __forceinline__ float abs_max4(float4 v, float m) {
    return fmaxf(m, fmaxf(fabsf(v.x), fmaxf(fabsf(v.y), fabsf(v.z))));
}

// Per-scene largest |component| of (dL/dX, dL/dV, dL/dE) as float bits
// (non-negative floats order like their bit patterns); NaN is kept as the
// largest value so that no scaling hides it. A block takes kGmaxPoints
// consecutive slots; a scene's points are one slot range, so a block whose
// first and last slots share a scene reduces in shared memory and issues
// one atomic (one per point on the same address was the kernel's cost),
// and a block across a scene boundary issues one per warp and scene.
constexpr int kGmaxThreads = 256;
constexpr int kGmaxPer = 8;
constexpr int kGmaxPoints = kGmaxThreads * kGmaxPer;

__device__ __forceinline__ uint32_t gmax_bits(const float4 a, const float4 b, const float4 c) {
    const float m = abs_max4(c, abs_max4(b, abs_max4(a, 0.0f)));
    const bool nan = isnan(a.x + a.y + a.z + b.x + b.y + b.z + c.x + c.y + c.z);
    return nan ? 0x7fffffffu : __float_as_uint(m);
}

__global__ void __launch_bounds__(kGmaxThreads)
k_adj_gmax(int n, const uint16_t *__restrict__ point_scene, const float4 *__restrict__ gx,
           const float4 *__restrict__ gv, const float4 *__restrict__ ge, uint32_t *__restrict__ gmax) {
    __shared__ uint32_t s_max[kGmaxThreads / 32];
    const int b0 = blockIdx.x * kGmaxPoints;
    const int last = min(b0 + kGmaxPoints, n) - 1;
    const unsigned lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    const uint32_t first_scene = point_scene ? point_scene[b0] : 0u;
    if (!point_scene || point_scene[last] == first_scene) {
        uint32_t bits = 0;
#pragma unroll
        for (int k = 0; k < kGmaxPer; k++) {
            const int i = b0 + k * kGmaxThreads + (int)threadIdx.x;
            if (i < n) bits = max(bits, gmax_bits(gx[i], gv[i], ge[i]));
        }
        bits = __reduce_max_sync(0xffffffffu, bits);
        if (lane == 0) s_max[w] = bits;
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t m = 0;
#pragma unroll
            for (int k = 0; k < kGmaxThreads / 32; k++) m = max(m, s_max[k]);
            if (m) atomicMax(&gmax[first_scene], m);
        }
        return;
    }
    for (int k = 0; k < kGmaxPer; k++) {   // across a scene boundary
        const int i = b0 + k * kGmaxThreads + (int)threadIdx.x;
        const bool valid = i < n;
        uint32_t bits = 0, scene = 0;
        if (valid) {
            bits = gmax_bits(gx[i], gv[i], ge[i]);
            scene = point_scene[i];
        }
        const uint32_t s0 = __shfl_sync(0xffffffffu, scene, 0);
        if (__all_sync(0xffffffffu, !valid || scene == s0)) {
            bits = __reduce_max_sync(0xffffffffu, bits);
            if (lane == 0 && bits) atomicMax(&gmax[s0], bits);
        } else if (valid && bits) {
            atomicMax(&gmax[scene], bits);
        }
    }
}

__device__ __forceinline__ int rescale_exponent(uint32_t bits) {
    const float m = __uint_as_float(bits);
    // at most 126, so that 2^-k stays a normal float
    return (bits < 0x7f800000u && m > kRescaleAbove) ? min(ilogbf(m), 126) : 0;
}

__global__ void __launch_bounds__(kThreads)
k_adj_rescale(int n, const uint16_t *__restrict__ point_scene, float4 *__restrict__ gx, float4 *__restrict__ gv,
              float4 *__restrict__ ge, const uint32_t *__restrict__ gmax) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int k = rescale_exponent(gmax[point_scene ? point_scene[i] : 0u]);
    if (!k) return;
    const float f = __int_as_float((127 - k) << 23);   // 2^-k, k in 40..126
    float4 a = gx[i], b = gv[i], c = ge[i];
    a.x *= f; a.y *= f; a.z *= f;
    b.x *= f; b.y *= f; b.z *= f;
    c.x *= f; c.y *= f; c.z *= f;
    gx[i] = a; gv[i] = b; ge[i] = c;
}

// The gradient itself from its mantissa: times 2^gexp (float; infinite
// where it overflows).
__global__ void __launch_bounds__(kThreads)
k_adj_apply_exponent(int n, const uint16_t *__restrict__ point_scene, float4 *__restrict__ gx,
                     float4 *__restrict__ gv, float4 *__restrict__ ge, const int *__restrict__ gexp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int k = gexp[point_scene ? point_scene[i] : 0u];
    if (!k) return;
    float4 a = gx[i], b = gv[i], c = ge[i];
    a.x = ldexpf(a.x, k); a.y = ldexpf(a.y, k); a.z = ldexpf(a.z, k);
    b.x = ldexpf(b.x, k); b.y = ldexpf(b.y, k); b.z = ldexpf(b.z, k);
    c.x = ldexpf(c.x, k); c.y = ldexpf(c.y, k); c.z = ldexpf(c.z, k);
    gx[i] = a; gv[i] = b; ge[i] = c;
}

__global__ void k_adj_bump(int nscenes, uint32_t *__restrict__ gmax, int *__restrict__ gexp) {
    const int sc = blockIdx.x * blockDim.x + threadIdx.x;
    if (sc >= nscenes) return;
    gexp[sc] += rescale_exponent(gmax[sc]);
    gmax[sc] = 0u;
}

// Identity tracking across recorded steps: out[s] = in[src[s]] (in null:
// out = src; src null: the identity).
__global__ void k_compose(int n, const uint32_t *__restrict__ src, const uint32_t *__restrict__ in,
                          uint32_t *__restrict__ out) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    out[s] = src ? (in ? in[src[s]] : src[s]) : (uint32_t)s;
}

// Up to three float4 arrays copied in one pass (tape saves and restores):
// dst_k[i] = src_k[i] for k < count.
struct Copy3 {
    const float4 *src[3];
    float4 *dst[3];
    int count;
};

__global__ void __launch_bounds__(kThreads) k_copy3(int n, const __grid_constant__ Copy3 c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    for (int k = 0; k < c.count; k++) c.dst[k][i] = c.src[k][i];
}

}  // namespace

// ---------------------------------------------------------------------------
// Launch wrappers.

int fl_launch_copy3(fl_system *s, int n, int count, const float4 *const *src, float4 *const *dst) {
    if (n == 0 || count == 0) return FL_OK;
    Copy3 c = {};
    c.count = count;
    for (int k = 0; k < count && k < 3; k++) { c.src[k] = src[k]; c.dst[k] = dst[k]; }
    k_copy3<<<blocks_for(n, kThreads), kThreads, 0, s->stream>>>(n, c);
    FL_LAUNCH_CHECK("copy3");
    return FL_OK;
}

static bool adj_prune(const fl_system *s) { return s->D.prune && s->codes_valid; }

int fl_launch_adj_advance(fl_system *s, const float *time_ptr, const float4 *force, const float4 *xo_b,
                          const float4 *vo_b, const float4 *eo_b, float4 *xa, float4 *ea, float4 *fb, float4 *v_out,
                          float2 *rr) {
    if (s->n == 0) return FL_OK;
    k_adj_advance<<<blocks_for(s->n, kAdjThreads), kAdjThreads, 0, s->stream>>>(
        s->D, fl_scene_tab(s), s->n, time_ptr, s->P.dt, s->f[F_GCELL].cur<uint32_t>(), s->src,
        s->f[F_POS].cur<float4>(), s->f[F_VEL].cur<float4>(), s->f[F_VEVAL].cur<float4>(),
        force, s->f[F_PRESS].cur<float>(), xo_b, vo_b, eo_b, xa, ea, fb, v_out, rr);
    FL_LAUNCH_CHECK("adj_advance");
    return FL_OK;
}

static int crowd_grid(const fl_system *s) { return 4 * s->num_sms; }

int fl_launch_adj_force(fl_system *s, const float2 *rr, const float4 *fb, float4 *xa, const float4 *ea, float *rb,
                        float4 *pc, float4 *e_out, uint32_t *revlist, uint32_t *revcnt, uint32_t *crowd,
                        uint32_t *crowd_count, uint32_t *revlong, uint32_t *revlong_count) {
    if (s->n == 0) return FL_OK;
    if (s->max_points > (int)kSlotMask)
        return fl_fail(FL_ERR_CAPACITY, "adjoint: %d points (at most %u)", s->max_points, kSlotMask);
    const bool pr = adj_prune(s);
    // the transposition saves work but adds three launches: it pays on
    // large systems, where the reverse step is bound by throughput
    const bool walk = s->adj_revmode == FL_REVERSE_WALK ||
                      (s->adj_revmode == FL_REVERSE_AUTO && s->n < FL_REVERSE_TRANSPOSE_MIN);
    if (walk) {
        auto walk = pr ? k_adj_revwalk<true> : k_adj_revwalk<false>;
        walk<<<blocks_for(s->n, kThreads), kThreads, grouping_smem(kThreads, kBandKeys), s->stream>>>(
            s->D, fl_scene_tab(s), s->n, s->f[F_POS].cur<float4>(), s->f[F_GCELL].cur<uint32_t>(), s->off, s->cnt,
            s->upbits, revlist, revcnt);
        FL_LAUNCH_CHECK("adj_revwalk");
    } else {
        FL_CUDA_TRY(cudaMemsetAsync(revcnt, 0, 4 * (size_t)s->n, s->stream));
        auto scatter = pr ? k_adj_revscatter<true> : k_adj_revscatter<false>;
        scatter<<<blocks_for(s->n, kThreads), kThreads, 0, s->stream>>>(
            s->D, fl_scene_tab(s), s->n, s->f[F_POS].cur<float4>(), s->f[F_GCELL].cur<uint32_t>(), s->off, s->cnt,
            s->upbits, s->hitlist, s->hitcnt, revlist, revcnt);
        FL_LAUNCH_CHECK("adj_revscatter");
        k_adj_revsort<<<blocks_for(s->n, kThreads), kThreads, 0, s->stream>>>(s->n, s->D.hcap, revlist, revcnt,
                                                                              revlong, revlong_count);
        FL_LAUNCH_CHECK("adj_revsort");
        auto listed = pr ? k_adj_revwalk_listed<true> : k_adj_revwalk_listed<false>;
        listed<<<crowd_grid(s), kThreads, 0, s->stream>>>(
            s->D, fl_scene_tab(s), s->f[F_POS].cur<float4>(), s->f[F_GCELL].cur<uint32_t>(), s->off, s->cnt,
            s->upbits, revlong, revlong_count, revlist, revcnt);
        FL_LAUNCH_CHECK("adj_revwalk_listed");
    }
    auto kern = pr ? k_adj_force<true> : k_adj_force<false>;
    kern<<<blocks_for(s->n, kAdjThreads), kAdjThreads, 0, s->stream>>>(
        s->D, fl_scene_tab(s), s->n, s->f[F_POS].cur<float4>(), s->f[F_VEVAL].cur<float4>(),
        rr, s->f[F_GCELL].cur<uint32_t>(), s->off, s->cnt, s->upbits, s->hitlist,
        s->hitcnt, s->src, fb, xa, ea, rb, pc, e_out, revlist, revcnt, CrowdList{crowd, crowd_count, (uint32_t)s->n});
    FL_LAUNCH_CHECK("adj_force");
    auto crowd_kern = pr ? k_adj_crowd_force<true> : k_adj_crowd_force<false>;
    crowd_kern<<<crowd_grid(s), kCrowdThreads, 0, s->stream>>>(
        s->D, fl_scene_tab(s), s->f[F_POS].cur<float4>(), s->f[F_VEVAL].cur<float4>(), rr,
        s->f[F_GCELL].cur<uint32_t>(), s->off, s->cnt, s->upbits, s->hitcnt, revcnt, s->src, fb, xa, e_out, rb, pc,
        CrowdList{crowd, crowd_count, (uint32_t)s->n});
    FL_LAUNCH_CHECK("adj_crowd_force");
    return FL_OK;
}

int fl_launch_adj_density(fl_system *s, const uint32_t *revlist, const uint32_t *revcnt, const float *rb,
                          const float4 *xa, float4 *x_out, uint32_t *crowd, uint32_t *crowd_count) {
    if (s->n == 0) return FL_OK;
    const bool pr = adj_prune(s);
    auto kern = pr ? k_adj_density<true> : k_adj_density<false>;
    kern<<<blocks_for(s->n, kAdjThreads), kAdjThreads, 0, s->stream>>>(
        s->D, fl_scene_tab(s), s->n, s->f[F_POS].cur<float4>(), s->f[F_GCELL].cur<uint32_t>(), s->off,
        s->cnt, s->upbits, s->hitlist, s->hitcnt, revlist, revcnt, s->src, rb, xa, x_out, false);
    FL_LAUNCH_CHECK("adj_density");
    auto crowd_kern = pr ? k_adj_crowd_density<true> : k_adj_crowd_density<false>;
    crowd_kern<<<crowd_grid(s), kCrowdThreads, 0, s->stream>>>(
        s->D, fl_scene_tab(s), s->f[F_POS].cur<float4>(), s->f[F_GCELL].cur<uint32_t>(), s->off, s->cnt, s->upbits,
        s->hitcnt, revcnt, s->src, rb, x_out, CrowdList{crowd, crowd_count, (uint32_t)s->n});
    FL_LAUNCH_CHECK("adj_crowd_density");
    return FL_OK;
}

int fl_param_chunks(int max_scene_points) {
    return max_scene_points <= 0 ? 1 : (max_scene_points + kReduceChunk - 1) / kReduceChunk;
}

int fl_launch_param_reduce(fl_system *s, const float4 *pc, const int *sbase, const int *sn, int nchunks,
                           double *partial, const int *gexp, double *acc) {
    if (s->n == 0) return FL_OK;
    dim3 grid((unsigned)nchunks, (unsigned)s->nscenes);
    k_param_partial<<<grid, kReduceThreads, 0, s->stream>>>(pc, sbase, sn, nchunks, partial);
    FL_LAUNCH_CHECK("param_partial");
    k_param_final<<<blocks_for(s->nscenes, 4), 128, 0, s->stream>>>(s->nscenes, nchunks, partial, gexp, acc);
    FL_LAUNCH_CHECK("param_final");
    return FL_OK;
}

int fl_launch_adj_apply_exponent(fl_system *s, float4 *gx, float4 *gv, float4 *ge, const int *gexp) {
    if (s->n == 0) return FL_OK;
    const uint16_t *ps = s->batched ? s->point_scene : nullptr;
    k_adj_apply_exponent<<<blocks_for(s->n, kThreads), kThreads, 0, s->stream>>>(s->n, ps, gx, gv, ge, gexp);
    FL_LAUNCH_CHECK("adj_apply_exponent");
    return FL_OK;
}

int fl_launch_adj_rescale(fl_system *s, float4 *gx, float4 *gv, float4 *ge, uint32_t *gmax, int *gexp) {
    if (s->n == 0) return FL_OK;
    const uint16_t *ps = s->batched ? s->point_scene : nullptr;
    k_adj_gmax<<<blocks_for(s->n, kGmaxPoints), kGmaxThreads, 0, s->stream>>>(s->n, ps, gx, gv, ge, gmax);
    FL_LAUNCH_CHECK("adj_gmax");
    k_adj_rescale<<<blocks_for(s->n, kThreads), kThreads, 0, s->stream>>>(s->n, ps, gx, gv, ge, gmax);
    FL_LAUNCH_CHECK("adj_rescale");
    k_adj_bump<<<blocks_for(s->nscenes, 128), 128, 0, s->stream>>>(s->nscenes, gmax, gexp);
    FL_LAUNCH_CHECK("adj_bump");
    return FL_OK;
}

int fl_launch_compose(fl_system *s, int n, const uint32_t *src, const uint32_t *in, uint32_t *out) {
    if (n == 0) return FL_OK;
    k_compose<<<blocks_for(n, kThreads), kThreads, 0, s->stream>>>(n, src, in, out);
    FL_LAUNCH_CHECK("compose");
    return FL_OK;
}

// k_force.cu -- pressure + artificial-viscosity acceleration and du/dt
// (sim/sph.go:327-401 AccelerationAndEDot2D) fused with the rest of the
// leapfrog step (sim/sph.go:121-193: kick, drift, periodic wrap,
// reflections). One thread per particle walks its k neighbours from the
// farthest to the nearest, as the reference's loop does, gathering the
// neighbours' predicted velocity, sound speed, density and smoothing length.
#include "physics.cuh"

#include <algorithm>

namespace sphgpu {

struct ForceArgs {
    Ctx c;
    PArrays B;  // positions / predictions of this evaluation (cell order)
    PArrays A;  // state written here (same order)
    Derived D;
    int integrate;
};

// sim/sph.go:121-193 with two roundings per multiply-add.
__device__ __forceinline__ void integrate_one(const SimDev &S, double2 &pos, double2 &vel, double &u,
                                              double ax, double ay, double udot) {
    const double dth = S.dth;
    const double dt2 = __dmul_rn(2.0, dth);
    vel.x = __dadd_rn(vel.x, __dmul_rn(ax, dt2));
    vel.y = __dadd_rn(vel.y, __dmul_rn(ay, dt2));
    u = __dadd_rn(u, __dmul_rn(__dmul_rn(udot, 2.0), dth));
    pos.x = __dadd_rn(pos.x, __dmul_rn(vel.x, dth));
    pos.y = __dadd_rn(pos.y, __dmul_rn(vel.y, dth));
    // periodic wrap: an if/continue chain, at most one axis per step
    if (pos.x < S.per_lo[0]) pos.x = __dadd_rn(pos.x, __dsub_rn(S.per_hi[0], S.per_lo[0]));
    else if (pos.x > S.per_hi[0]) pos.x = __dsub_rn(pos.x, __dsub_rn(S.per_hi[0], S.per_lo[0]));
    else if (pos.y < S.per_lo[1]) pos.y = __dadd_rn(pos.y, __dsub_rn(S.per_hi[1], S.per_lo[1]));
    else if (pos.y > S.per_hi[1]) pos.y = __dsub_rn(pos.y, __dsub_rn(S.per_hi[1], S.per_lo[1]));
    // reflections: Pos -= Pos - bound; Vel = -Vel
    if (pos.x < S.refl[0]) { pos.x = __dsub_rn(pos.x, __dsub_rn(pos.x, S.refl[0])); vel.x = -vel.x; }
    if (pos.x > S.refl[1]) { pos.x = __dsub_rn(pos.x, __dsub_rn(pos.x, S.refl[1])); vel.x = -vel.x; }
    if (pos.y < S.refl[2]) { pos.y = __dsub_rn(pos.y, __dsub_rn(pos.y, S.refl[2])); vel.y = -vel.y; }
    if (pos.y > S.refl[3]) { pos.y = __dsub_rn(pos.y, __dsub_rn(pos.y, S.refl[3])); vel.y = -vel.y; }
}

// The mixed form (the FP64 forms run k_force_fp64 below).
template <int MODE>
__global__ void __launch_bounds__(256, 4) k_force(ForceArgs a) {
    static_assert(MODE == MODE_MIXED, "the FP64 forms run k_force_fp64");
    const int k = a.c.k;
    const PArrays &B = a.B;
    const Derived &D = a.D;
    unsigned fl = 0;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < a.c.n;
         q += (int64_t)gridDim.x * blockDim.x) {
        const int s = sim_of(a.c, q);
        const SimDev &S = a.c.sims[s];
        const double2 P = B.pos[q];
        const int32_t *nb = D.nbr + q * k;
        double axo, ayo, edot;
        {
            // FP32 throughout the sums and prefactors (no FP64 work per particle
            // before the integrator)
            const float4 di = D.derf[q];
            const float ci = di.x, rhoi = di.y, hif = di.z, caf = di.w;
            const float inv_hf = 1.f / hif;
            const float4 pr = B.rec[q];
            const float4 vi = B.vrec[q];
            const float alpha = S.falpha, beta = S.fbeta, etasq = S.fetasq;
            KahanF ax, ay, ed;
            auto pair = [&](uint32_t code) {
                const uint32_t j = code >> kCodeShift;
                float rabx, raby;  // r_AB = (q - offset) - p from float pairs
                float_pair_rel(S, pr, __ldg(&B.rec[j]), code & 15u, rabx, raby);
                const float d2 = __fmaf_rn(rabx, rabx, raby * raby);
                const float invd = rsqrtf(d2);
                const float qq = fminf(d2 * invd * inv_hf, 1.f);
                const float drk = kdf_f32(S.kernel, qq);
                const float4 vj = __ldg(&B.vrec[j]);
                const float4 dj = __ldg(&D.derf[j]);
                const float vabx = (vj.x - vi.x) + (vj.z - vi.z);
                const float vaby = (vj.y - vi.y) + (vj.w - vi.w);
                const float dot = vabx * rabx + vaby * raby;
                float piab = 0.f;
                if (dot < 0.f) {
                    const float cab = 0.5f * (ci + dj.x);
                    const float rhoab = 0.5f * (rhoi + dj.y);
                    const float hab = 0.5f * (hif + dj.z);
                    // two-instruction quotients (<= 2 ulp; both denominators are
                    // normal: d2 + eta^2 >= eta^2, rho_AB > 0)
                    const float mu = __fdividef(dot * hab, d2 + etasq);
                    piab = __fdividef(mu * (beta * mu - alpha * cab), rhoab);
                }
                const float w = (piab + caf + dj.w) * drk * invd;
                ax.add(rabx * w);
                ay.add(raby * w);
                ed.add(dot * drk);
            };
            for_each_nbr_desc(nb, k, [&](int, uint32_t code) { pair(code); });
            const float ff = S.fdfm * (inv_hf * inv_hf * inv_hf);
            axo = (double)(ax.value_f() * ff) + S.accel[0];
            ayo = (double)(ay.value_f() * ff) + S.accel[1];
            edot = (double)(caf * ed.value_f() * S.fmass);
        }
        if (!isfinite(axo) || !isfinite(ayo) || !isfinite(edot)) fl |= FLAG_Q_RANGE;
        double2 pos = P, vel = B.vel[q];
        double u = B.u[q];
        if (a.integrate) integrate_one(S, pos, vel, u, axo, ayo, edot);
        a.A.pos[q] = pos;
        a.A.vel[q] = vel;
        a.A.u[q] = u;
        a.A.acc[q] = make_double2(axo, ayo);
        a.A.udot[q] = edot;
        a.A.id[q] = B.id[q];
        a.A.hprev[q] = (float)D.h[q];
        a.A.vp[q] = B.vp[q];
        a.A.up[q] = B.up[q];
    }
    if (fl) atomicOr(a.c.flags, fl);
}

// ---------------------------------------------------------------- FP64 form,
// viscosity compacted. One warp per 32 consecutive particles, one lane per
// particle, in three phases:
//   1. each lane flags its approaching neighbour pairs (v_AB . r_AB < 0);
//   2. the warp computes the viscosity term Pi of every flagged pair of its
//      32 particles with all lanes busy (the pairs dealt out in turn) and
//      keeps them in shared memory;
//   3. each lane sums its k terms farthest first (sim/sph.go:343-392), taking
//      Pi from shared memory for the flagged pairs.
// Phase 3 is the reference's loop with Pi looked up instead of computed in a
// branch that a warp runs whenever any of its lanes needs it; every operation
// and its order are unchanged, so the results stay bit-exact.
constexpr int kForceWarps = 4;

// per-warp shared memory: Pi doubles of one chunk (at most 32 entries per
// particle), masks, counts; rounded up to 16 bytes so that every warp's Pi
// array starts 8-byte (in fact 16-byte) aligned
__host__ __device__ constexpr size_t force_exact_warp_bytes(int k) {
    return ((size_t)(k < 32 ? k : 32) * 256 + 4 * 32 * 4 + 33 * 4 + 15) & ~(size_t)15;
}
constexpr bool force_exact_layout_aligned() {
    for (int k = 1; k <= 128; k++)
        if (force_exact_warp_bytes(k) % 16 != 0 || ((size_t)k * 256) % 8 != 0) return false;
    return true;
}
static_assert(force_exact_layout_aligned(), "per-warp shared-memory regions must stay 16-byte aligned");

// r_AB = (q - offset) - p and v_AB . r_AB for neighbour code `code` of a
// particle at P with predicted velocity vpi (sim/sph.go:355-367)
__device__ __forceinline__ void pair_geom(const SimDev &S, const PArrays &B, uint32_t code, double2 P, double2 vpi,
                                          double &rabx, double &raby, double &dot) {
    const uint32_t j = code >> kCodeShift;
    const double2 vpj = B.vp[j];
    const double vabx = __dsub_rn(vpj.x, vpi.x), vaby = __dsub_rn(vpj.y, vpi.y);
    const double2 Q = B.pos[j];
    if ((code & 15u) == 4u) {  // q - 0 = q exactly
        rabx = __dsub_rn(Q.x, P.x);
        raby = __dsub_rn(Q.y, P.y);
    } else {
        double ox, oy;
        img_shift(S, code & 15u, ox, oy);
        rabx = __dsub_rn(__dsub_rn(Q.x, ox), P.x);
        raby = __dsub_rn(__dsub_rn(Q.y, oy), P.y);
    }
    dot = __dadd_rn(emu_mul_ol(vabx, rabx), emu_mul_ol(vaby, raby));
}

template <int MODE>
__global__ void __launch_bounds__(kForceWarps * 32) k_force_fp64(ForceArgs a) {
    static_assert(MODE == MODE_EXACT64 || MODE == MODE_FAST64, "FP64 forms only");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int k = a.c.k;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int nw = (k + 31) >> 5;  // mask words per particle (k <= 128)
    // per warp: Pi[min(k, 32)][32] doubles, approach masks [4][32], inclusive pair counts [33]
    unsigned char *wb = smem_raw + (size_t)w * force_exact_warp_bytes(k);
    double *spi = (double *)wb;
    uint32_t *smask = (uint32_t *)(wb + (size_t)(k < 32 ? k : 32) * 256);
    int32_t *sinc = (int32_t *)(smask + 4 * 32);
    const PArrays &B = a.B;
    const Derived &D = a.D;
    unsigned fl = 0;
    const int64_t n = a.c.n;
    for (int64_t q0 = ((int64_t)blockIdx.x * kForceWarps + w) * 32; q0 < n;
         q0 += (int64_t)gridDim.x * kForceWarps * 32) {
        const int64_t q = q0 + lane;
        const bool valid = q < n;
        const SimDev &S = a.c.sims[valid ? sim_of(a.c, q) : 0];
        double2 P = make_double2(0.0, 0.0), vpi = P;
        double4 di = make_double4(0.0, 0.0, 0.0, 0.0);
        const int32_t *nb = D.nbr + q * k;
        // ---- 1. approaching pairs: the sign of v_AB . r_AB from the float-pair
        // records, with an error bound; the reference's FP64 dot product only
        // where the bound cannot decide (e.g. equal velocities)
        if (valid) {
            P = B.pos[q];
            vpi = B.vp[q];
            di = D.der[q];
            const float4 pr = B.rec[q], vi = B.vrec[q];
            const float dXh = S.fimg_h[0], dXl = S.fimg_l[0], dYh = S.fimg_h[1], dYl = S.fimg_l[1];
            const float lbig = 2.f * fmaxf(S.flmax, S.fmag);
            uint32_t m0 = 0, m1 = 0, m2 = 0, m3 = 0;  // approach bits of entries 0-31, 32-63, ...
            for_each_nbr_desc(nb, k, [&](int e, uint32_t code) {
                {
                    const uint32_t j = code >> kCodeShift;
                    const int ia = (int)((code & 15u) / 3u) - 1, ib = (int)((code & 15u) % 3u) - 1;
                    const float4 r = B.rec[j], vj = B.vrec[j];
                    const float rx = ((r.x - (ia > 0 ? dXh : 0.f)) - (ia < 0 ? pr.x - dXh : pr.x)) +
                                     (r.z - (pr.z + (ia > 0 ? dXl : ia < 0 ? -dXl : 0.f)));
                    const float ry = ((r.y - (ib > 0 ? dYh : 0.f)) - (ib < 0 ? pr.y - dYh : pr.y)) +
                                     (r.w - (pr.w + (ib > 0 ? dYl : ib < 0 ? -dYl : 0.f)));
                    const float vx = (vj.x - vi.x) + (vj.z - vi.z), vy = (vj.y - vi.y) + (vj.w - vi.w);
                    const float px = vx * rx, py = vy * ry;
                    const float dotf = px + py;
                    // |dotf - reference dot| bound: float-pair residues (2^-48 relative
                    // to |p|, |v|), FP32 differences, products and sum (2^-23 each)
                    const float vmag = fabsf(vj.x) + fabsf(vi.x) + fabsf(vj.y) + fabsf(vi.y);
                    const float eb = 9.5367431640625e-7f * (fabsf(px) + fabsf(py)) +
                                     9.094947017729282e-13f * (lbig * (fabsf(vx) + fabsf(vy)) + vmag * (fabsf(rx) + fabsf(ry)));
                    bool approach;
                    if (dotf < -eb) approach = true;
                    else if (dotf > eb) approach = false;
                    else {
                        double rabx, raby, dot;
                        pair_geom(S, B, code, P, vpi, rabx, raby, dot);
                        approach = dot < 0.0;
                    }
                    if (approach) {
                        const uint32_t bit = 1u << (e & 31);
                        if (e < 32) m0 |= bit;
                        else if (e < 64) m1 |= bit;
                        else if (e < 96) m2 |= bit;
                        else m3 |= bit;
                    }
                }
            });
            const uint32_t mw[4] = {m0, m1, m2, m3};
#pragma unroll
            for (int wd = 0; wd < 4; wd++) {
                if (wd < nw) {
                    smask[wd * 32 + lane] = mw[wd];
                }
            }
        } else {
            for (int wd = 0; wd < nw; wd++) smask[wd * 32 + lane] = 0u;
        }
        // ---- 2 and 3 one chunk of 32 neighbour entries at a time (the chunk
        // of mask word c: entries 32 c .. 32 c + 31), farthest chunk first, so
        // the Pi table holds 32 entries per particle whatever k is; the sums run
        // through the chunks in the reference's order (sim/sph.go:343,
        // farthest first)
        const double ca = di.w;
        const double2 *dist = D.dist + q * k;
        double ax = 0.0, ay = 0.0, ed = 0.0;
        for (int c = nw - 1; c >= 0; c--) {
            const int e_lo = 32 * c, e_hi = min(k, e_lo + 32);
            const uint32_t mine = smask[c * 32 + lane];
            int inc = __popc(mine);
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, inc, o);
                if (lane >= o) inc += y;
            }
            sinc[lane] = inc;
            const int total = __shfl_sync(0xffffffffu, inc, 31);
            __syncwarp();
            // ---- 2. Pi of every flagged pair of the chunk
            for (int i = lane; i < total; i += 32) {
                int p = 0;  // owner: the first lane whose inclusive count exceeds i
#pragma unroll
                for (int b = 16; b > 0; b >>= 1)
                    if (sinc[p + b - 1] <= i) p += b;
                const int r = i - (p ? sinc[p - 1] : 0);  // r-th flagged pair of particle p in the chunk
                uint32_t m = smask[c * 32 + p];
                for (int t = 0; t < r; t++) m &= m - 1;
                const int eo = __ffs(m) - 1;  // entry e_lo + eo
                const int64_t qp = q0 + p;
                const SimDev &Sp = a.c.sims[sim_of(a.c, qp)];
                const double2 Pp = B.pos[qp], vpp = B.vp[qp];
                const double4 dp = D.der[qp];
                const uint32_t code = (uint32_t)D.nbr[qp * k + e_lo + eo];
                double rabx, raby, dot;
                pair_geom(Sp, B, code, Pp, vpp, rabx, raby, dot);
                const double4 dj = D.der[code >> kCodeShift];
                if (MODE == MODE_EXACT64) {
                    const double cab = __dmul_rn(0.5, __dadd_rn(dp.x, dj.x));
                    const double rhoab = __dmul_rn(0.5, __dadd_rn(dp.y, dj.y));
                    const double hab = __dmul_rn(0.5, __dadd_rn(dp.z, dj.z));
                    const double r2 = __dadd_rn(__dmul_rn(rabx, rabx), __dmul_rn(raby, raby));
                    const double den = __dadd_rn(r2, Sp.etasq);
                    const double mu = emu_div_ol(emu_mul_ol(dot, hab), emu_divisor_ol(den), den);
                    spi[eo * 32 + p] = emu_div_ol(__dadd_rn(emu_mul_ol(emu_mul_ol(-Sp.alpha, cab), mu),
                                                            emu_mul_ol(emu_mul_ol(Sp.beta, mu), mu)),
                                                  emu_divisor_ol(rhoab), rhoab);
                } else {
                    const double cab = 0.5 * (dp.x + dj.x), rhoab = 0.5 * (dp.y + dj.y), hab = 0.5 * (dp.z + dj.z);
                    const double mu = dot * hab / (rabx * rabx + raby * raby + Sp.etasq);
                    spi[eo * 32 + p] = mu * (Sp.beta * mu - Sp.alpha * cab) / rhoab;
                }
            }
            __syncwarp();
            // ---- 3. the chunk's terms of the reference's ordered sums
            if (valid) {
                if (MODE == MODE_EXACT64) {
                    for_each_nbr_desc_range(nb, e_lo, e_hi, k, [&](int e, uint32_t code) {
                        const double d = dist[e].x;
                        const double drk = dist[e].y;  // dF(NNDists[i]/maxR), evaluated by the density pass
                        double rabx, raby, dot;
                        pair_geom(S, B, code, P, vpi, rabx, raby, dot);
                        const bool visc = (mine >> (e - e_lo)) & 1u;
                        const double piab = visc ? spi[(e - e_lo) * 32 + lane] : 0.0;
                        const double cb = D.der[code >> kCodeShift].w;
                        const double sum3 = __dadd_rn(__dadd_rn(piab, ca), cb);
                        // both quotients by NNDists[i] share one prepared divisor
                        const EmuDivisor dd = emu_divisor_ol(d);
                        ax = __dadd_rn(ax, emu_div_ol(emu_mul_ol(emu_mul_ol(rabx, sum3), drk), dd, d));
                        ay = __dadd_rn(ay, emu_div_ol(emu_mul_ol(emu_mul_ol(raby, sum3), drk), dd, d));
                        ed = __dadd_rn(ed, emu_mul_ol(dot, drk));
                    });
                } else {
                    // the fast form keeps (dF, dF / NNDists) per neighbour
                    for_each_nbr_desc_range(nb, e_lo, e_hi, k, [&](int e, uint32_t code) {
                        const double2 dd = dist[e];
                        const uint32_t j = code >> kCodeShift;
                        const double2 vpj = B.vp[j], Q = B.pos[j];
                        double ox = 0.0, oy = 0.0;
                        if ((code & 15u) != 4u) img_shift(S, code & 15u, ox, oy);
                        const double rabx = (Q.x - ox) - P.x, raby = (Q.y - oy) - P.y;
                        const double dot = (vpj.x - vpi.x) * rabx + (vpj.y - vpi.y) * raby;
                        const bool visc = (mine >> (e - e_lo)) & 1u;
                        const double piab = visc ? spi[(e - e_lo) * 32 + lane] : 0.0;
                        const double w = (piab + ca + D.der[j].w) * dd.y;
                        ax += rabx * w;
                        ay += raby * w;
                        ed += dot * dd.x;
                    });
                }
            }
            __syncwarp();
        }
        if (valid) {
            const double hi = di.z;
            double axo, ayo, edot;
            if (MODE == MODE_EXACT64) {
                const double f = __ddiv_rn(__dmul_rn(S.mass, S.dfpref), __dmul_rn(__dmul_rn(hi, hi), hi));
                axo = __dadd_rn(__dmul_rn(ax, f), S.accel[0]);
                ayo = __dadd_rn(__dmul_rn(ay, f), S.accel[1]);
                edot = __dmul_rn(__dmul_rn(ca, ed), S.mass);
            } else {
                const double inv_h = 1.0 / hi;
                const double f = S.mass * S.dfpref * (inv_h * inv_h * inv_h);
                axo = ax * f + S.accel[0];
                ayo = ay * f + S.accel[1];
                edot = ca * ed * S.mass;
            }
            if (!isfinite(axo) || !isfinite(ayo) || !isfinite(edot)) fl |= FLAG_Q_RANGE;
            double2 pos = P, vel = B.vel[q];
            double u = B.u[q];
            if (a.integrate) integrate_one(S, pos, vel, u, axo, ayo, edot);
            a.A.pos[q] = pos;
            a.A.vel[q] = vel;
            a.A.u[q] = u;
            a.A.acc[q] = make_double2(axo, ayo);
            a.A.udot[q] = edot;
            a.A.id[q] = B.id[q];
            a.A.hprev[q] = (float)D.h[q];
            a.A.vp[q] = vpi;
            a.A.up[q] = B.up[q];
        }
        __syncwarp();
    }
    if (fl) atomicOr(a.c.flags, fl);
}

static size_t force_exact_smem(int k) { return (size_t)kForceWarps * force_exact_warp_bytes(k); }

static int g_force_exact_blocks[129];  // resident blocks per SM by k (filled before any capture)

// Sets the shared-memory limit of the FP64 force kernel and records its
// occupancy for k; must run before any stream capture.
void force_init_attrs(int k) {
    cudaFuncSetAttribute(k_force_fp64<MODE_EXACT64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)force_exact_smem(128));
    cudaFuncSetAttribute(k_force_fp64<MODE_FAST64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)force_exact_smem(128));
    if (k >= 1 && k <= 128 && !g_force_exact_blocks[k]) {
        int nb = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, k_force_fp64<MODE_EXACT64>, kForceWarps * 32, force_exact_smem(k));
        g_force_exact_blocks[k] = std::max(nb, 1);
    }
}

void launch_force(const Ctx &c, const Launch &L, const PArrays &B, const PArrays &A,
                  const Derived &D, int mode, bool integrate) {
    ForceArgs a;
    a.c = c;
    a.B = B;
    a.A = A;
    a.D = D;
    a.integrate = integrate ? 1 : 0;
    const int block = 128;
    int64_t need = (c.n + block - 1) / block;
    int grid = (int)(need < (int64_t)L.sms * 16 ? need : (int64_t)L.sms * 16);
    if (grid < 1) grid = 1;
    if (mode == MODE_EXACT64 || mode == MODE_FAST64) {
        const int64_t tiles = (c.n + 31) / 32;
        const int64_t eneed = (tiles + kForceWarps - 1) / kForceWarps;
        const int nb = c.k >= 1 && c.k <= 128 ? std::max(g_force_exact_blocks[c.k], 1) : 1;
        const int eg = (int)std::max<int64_t>(1, std::min<int64_t>(eneed, (int64_t)L.sms * nb));
        if (mode == MODE_EXACT64) k_force_fp64<MODE_EXACT64><<<eg, kForceWarps * 32, force_exact_smem(c.k), L.stream>>>(a);
        else k_force_fp64<MODE_FAST64><<<eg, kForceWarps * 32, force_exact_smem(c.k), L.stream>>>(a);
    }
    else k_force<MODE_MIXED><<<grid, block, 0, L.stream>>>(a);
}

// ------------------------------------------------------------ error norms
// Per particle, the sums of the magnitudes of its neighbour terms in the
// acceleration and in du/dt: the normalisers of the mixed form's error
// statements. Read from the FP64 form's last evaluation (positions, predicted
// velocities, lists with (NNDists, dF), per-particle (c, rho, h, c^2/(gamma
// rho))), in the reference's term order (sim/sph.go:343-392, farthest first)
// and rounding, so that they equal the oracle's norms bit for bit.
__global__ void k_error_norms(Ctx c, PArrays B, Derived D, double *anorm, double *unorm) {
    const int k = c.k;
    for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < c.n;
         q += (int64_t)gridDim.x * blockDim.x) {
        const SimDev &S = c.sims[sim_of(c, q)];
        const double2 P = B.pos[q], vpi = B.vp[q];
        const double4 di = D.der[q];  // (c, rho, h, c^2/(gamma rho))
        const int32_t *nb = D.nbr + q * k;
        const double2 *dist = D.dist + q * k;
        double an = 0.0, un = 0.0;
        for (int e = k - 1; e >= 0; e--) {
            const uint32_t code = (uint32_t)nb[e];
            double rabx, raby, dot;
            pair_geom(S, B, code, P, vpi, rabx, raby, dot);
            const double d = dist[e].x, drk = dist[e].y;
            const double4 dj = D.der[code >> kCodeShift];
            double piab = 0.0;
            if (dot < 0.0) {
                const double cab = __dmul_rn(0.5, __dadd_rn(di.x, dj.x));
                const double rhoab = __dmul_rn(0.5, __dadd_rn(di.y, dj.y));
                const double hab = __dmul_rn(0.5, __dadd_rn(di.z, dj.z));
                const double r2 = __dadd_rn(__dmul_rn(rabx, rabx), __dmul_rn(raby, raby));
                const double mu = __ddiv_rn(__dmul_rn(dot, hab), __dadd_rn(r2, S.etasq));
                piab = __ddiv_rn(__dadd_rn(__dmul_rn(__dmul_rn(-S.alpha, cab), mu), __dmul_rn(__dmul_rn(S.beta, mu), mu)),
                                 rhoab);
            }
            const double w = __ddiv_rn(__dmul_rn(__dadd_rn(__dadd_rn(piab, di.w), dj.w), drk), d);
            an = __dadd_rn(an, __dmul_rn(__dsqrt_rn(__dadd_rn(__dmul_rn(rabx, rabx), __dmul_rn(raby, raby))), fabs(w)));
            un = __dadd_rn(un, fabs(__dmul_rn(dot, drk)));
        }
        const double f = __ddiv_rn(__dmul_rn(S.mass, S.dfpref), __dmul_rn(__dmul_rn(di.z, di.z), di.z));
        const int32_t id = B.id[q];
        anorm[id] = __dmul_rn(an, fabs(f));
        unorm[id] = __dmul_rn(un, fabs(__dmul_rn(di.w, S.mass)));
    }
}

void launch_error_norms(const Ctx &c, const Launch &L, const PArrays &B, const Derived &D, double *anorm,
                        double *unorm) {
    const int block = 256;
    const int64_t need = (c.n + block - 1) / block;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(need, (int64_t)L.sms * 8));
    k_error_norms<<<grid, block, 0, L.stream>>>(c, B, D, anorm, unorm);
}

}  // namespace sphgpu

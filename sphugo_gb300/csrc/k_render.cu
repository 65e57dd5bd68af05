// k_render.cu -- frame rasteriser: the reference's CPU animator frame
// (sim/animator.go:55-103 CurrentFrame) as two CUDA kernels writing a headless
// NRGBA buffer instead of an OpenGL window.
//
// The reference sorts particles by -Z (sim/heap.go:229-268 QuickSort) and
// paints a disk of radius 4 pixels for each in that order
// (gx/graphics.go:90-107 DrawDisk), coloured by ParaRamp
// (gx/graphics.go:156-164) of min(rho / (m N 10) * 256, 255). Painting in order
// means every pixel shows the LAST disk that covers it, so here each particle
// raises the pixels it covers to its draw rank with atomicMax (k_draw), and a
// second pass colours each pixel from the winning particle's density
// (k_resolve). Pixel tests keep the reference's FP32 arithmetic and rounding
// (no contraction), so frames are identical to a sequential painter.
#include "physics.cuh"

namespace sphgpu {

__constant__ uchar4 c_ramp[256];

#define GRID_STRIDE(i, n) \
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < (n); i += (int64_t)gridDim.x * blockDim.x)

__global__ void k_draw(Ctx c, PArrays A, const int32_t *zrank, int32_t *rslot, int32_t *fb, int W, int H) {
    GRID_STRIDE(i, c.n) {
        const int32_t id = A.id[i];
        const int32_t r = zrank ? zrank[id] : id;  // default: caller order, the last on top
        rslot[r] = (int32_t)i;
        const double2 p = A.pos[i];
        // x := float32(Pos.X) * float32(W)
        const float cx = __fmul_rn(__double2float_rn(p.x), (float)W);
        const float cy = __fmul_rn(__double2float_rn(p.y), (float)H);
        const float rad = 4.f;
        const float fxa = floorf(__fsub_rn(cx, rad)), fxb = ceilf(__fadd_rn(cx, rad));
        const float fya = floorf(__fsub_rn(cy, rad)), fyb = ceilf(__fadd_rn(cy, rad));
        // pixels outside the canvas are ignored (image.NRGBA.Set); NaN positions draw nothing
        if (!(fxb >= 0.f && fxa <= (float)(W - 1) && fyb >= 0.f && fya <= (float)(H - 1))) continue;
        const int xa = max((int)fxa, 0), xb = min((int)fxb, W - 1);
        const int ya = max((int)fya, 0), yb = min((int)fyb, H - 1);
        for (int x = xa; x <= xb; x++) {
            const float dx = __fsub_rn((float)x, cx);
            const float dx2 = __fmul_rn(dx, dx);
            for (int y = ya; y <= yb; y++) {
                const float dy = __fsub_rn((float)y, cy);
                if (__fadd_rn(dx2, __fmul_rn(dy, dy)) <= __fmul_rn(rad, rad)) atomicMax(&fb[(int64_t)y * W + x], r);
            }
        }
    }
}

__global__ void k_resolve(const int32_t *fb, const int32_t *rslot, const double *rho, int64_t n_eval, double mass,
                          double n10, uchar4 *out, int64_t npix) {
    GRID_STRIDE(p, npix) {
        const int32_t r = fb[p];
        uchar4 col = make_uchar4(0, 0, 0, 255);  // gx.BLACK
        if (r >= 0) {
            const int32_t s = rslot[r];
            const double rh = s < n_eval ? rho[s] : 0.0;
            // float64(Rho / (m * float64(N*10)) * 256), then uint8(math.Min(., 255))
            const double cf = __dmul_rn(__ddiv_rn(rh, __dmul_rn(mass, n10)), 256.0);
            const double mn = cf > 255.0 ? 255.0 : cf;  // math.Min keeps a NaN
            const int idx = mn >= 0.0 ? (int)mn : 0;    // uint8(): truncation; NaN gives 0
            col = c_ramp[idx];
        }
        out[p] = col;
    }
}

int set_ramp(const unsigned char rgba[256 * 4]) {
    return cudaMemcpyToSymbol(c_ramp, rgba, 256 * 4) == cudaSuccess ? 0 : -1;
}

void launch_render(const Ctx &c, const Launch &L, const PArrays &A, const int32_t *zrank, int32_t *rslot,
                   int32_t *fb, const double *rho, int64_t n_eval, double mass, int W, int H, uchar4 *out) {
    const int64_t npix = (int64_t)W * H;
    cudaMemsetAsync(fb, 0xff, npix * sizeof(int32_t), L.stream);  // -1: no disk
    const int64_t pg = std::min<int64_t>((c.n + 127) / 128, (int64_t)L.sms * 16);
    k_draw<<<(int)std::max<int64_t>(pg, 1), 128, 0, L.stream>>>(c, A, zrank, rslot, fb, W, H);
    const int64_t rg = std::min<int64_t>((npix + 255) / 256, (int64_t)L.sms * 16);
    k_resolve<<<(int)std::max<int64_t>(rg, 1), 256, 0, L.stream>>>(fb, rslot, rho, n_eval, mass,
                                                                   (double)(c.n * 10), out, npix);
}

}  // namespace sphgpu

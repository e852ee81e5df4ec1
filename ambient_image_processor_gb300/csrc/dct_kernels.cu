// DCT-II / DCT-III Poisson integration of the bias gradient field v.
//
// The reference integrates v with four host round trips (divergence, DCT, Poisson
// division, inverse DCT), and evaluates each separable DCT pass as one thread per
// output voxel looping over the whole line with an FP64 cospi per term
// (cuda_image_operations/cosine_transform.cu:142-223, inverse_cosine_transform.cu:79-164).
// Here each separable pass is a batched matrix contraction of the volume with an
// N x N cosine matrix, everything stays on the device, the divergence of v is
// computed inside the first pass's operand load, and the Poisson eigenvalue
// division is the epilogue of the last forward pass.
//
// A pass along axis a contracts the a-index of the volume with a matrix M:
//   x (contiguous lines):   out[r][k]    = sum_n in[r][n]    M[k][n]   r = z*H + y
//   y (batched over z):     out[z][k][x] = sum_n M[k][n] in[z][n][x]
//   z:                      out[k][t]    = sum_n M[k][n] in[n][t]      t = y*W + x
// M is the DCT-II matrix C[k][n] = cospi((n + 1/2) k / N) for the forward passes and
// the DCT-III matrix S[m][k] = w_k cospi((m + 1/2) k / N), w_0 = 1, w_k = 2, for the
// inverse passes.  Forward x8 and inverse /(8 W H D) follow the reference's scale
// factors (cosine_transform.cu:222, inverse_cosine_transform.cu:163), so the round
// trip is the identity.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"

namespace tgvdct {

namespace {

double cospi_host(double a) {
    double r = std::fmod(std::fabs(a), 2.0);
    if (r > 1.0) r = 2.0 - r;
    const double pi = 3.14159265358979323846;
    if (r <= 0.25) return std::cos(pi * r);
    if (r <= 0.75) return std::sin(pi * (0.5 - r));
    return -std::cos(pi * (1.0 - r));
}

size_t a256(size_t b) { return (b + 255) & ~size_t(255); }

__global__ void cosk_kernel(float* out, int N) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < N) out[k] = cospif((float)k / (float)N);  // solve_poisson_in_cosine_domain.cu:48-53
}

// fx[k] = 2 cosk[k] * 2^32 as an integer; raises *inexact where the float is not an
// integer multiple of 2^-32 (then the plan keeps the FP64 form)
__global__ void cosk_fx_kernel(const float* cosk, int N, long long* fx, int* inexact) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= N) return;
    const float v = cosk[k] * 8589934592.f;  // 2^33: exact scaling
    const long long t = __float2ll_rn(v);
    fx[k] = t;
    if ((float)t != v) atomicExch(inexact, 1);
}

// ---- batched SIMT contraction ------------------------------------------------------
constexpr int TM = 64, TN = 64, TK = 16, NT = 256;

enum Epilogue { EPI_NONE = 0, EPI_SCALE = 1, EPI_POISSON_REF = 2, EPI_POISSON_ACC = 3 };
enum ALoad { A_PLAIN = 0, A_DIVERGENCE = 1 };

struct GemmArgs {
    int M, N, K;
    const float* A;
    long long sAi, sAk, sAb;
    const float* B;
    long long sBk, sBj, sBb;
    float* C;
    long long sCi, sCj, sCb;
    // A_DIVERGENCE: A[i][k] = (B_x v_x + B_y v_y (+ B_z v_z)) at voxel x = k, row i
    const float* vx;
    const float* vy;
    const float* vz;
    int W, H, D;
    // epilogue
    float scale;
    int pz_layout;  // 1: outputs indexed (i = ky, j = kx); 2: (i = kz, j = ky*W + kx)
    long long col_off;  // layout 2 on a pencil: the global index of output column j = 0
    const long long* fx0;  // DctPlan::cosk_fx (null: the FP64 form)
    const long long* fx1;
    const long long* fx2;
    const float* cosk0;
    const float* cosk1;
    const float* cosk2;
    const float* eig0;
    const float* eig1;
    const float* eig2;
};

__device__ __forceinline__ float div_at(const GemmArgs& g, int i, int k) {
    // voxel (x = k, y = i % H, z = i / H)
    const int y = i % g.H, z = i / g.H;
    const size_t W = (size_t)g.W, WH = (size_t)g.W * g.H;
    const size_t idx = (size_t)i * W + k;
    const float bx = (k > 0 ? g.vx[idx - 1] : 0.f) - g.vx[idx];   // divergence.cu:38-55
    const float by = (y > 0 ? g.vy[idx - W] : 0.f) - g.vy[idx];
    float s = bx + by;
    if (g.D > 1) s = s + ((z > 0 ? g.vz[idx - WH] : 0.f) - g.vz[idx]);
    return s;
}

template <int ALOAD, int EPI>
__global__ void __launch_bounds__(NT) gemm_kernel(GemmArgs g) {
    __shared__ float As[TK][TM + 4];
    __shared__ float Bs[TK][TN + 4];
    const int b = blockIdx.z;
    const int i0 = blockIdx.y * TM, j0 = blockIdx.x * TN;
    const int t = threadIdx.x;
    const int ti = t / 16, tj = t % 16;  // 16 x 16 threads, 4 x 4 outputs each
    const float* A = g.A + (long long)b * g.sAb;
    const float* B = g.B + (long long)b * g.sBb;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < g.K; k0 += TK) {
        // A tile: TM x TK
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int e = t + r * NT;
            int ii, kk;
            if (g.sAk == 1 || ALOAD == A_DIVERGENCE) { kk = e % TK; ii = e / TK; }
            else { ii = e % TM; kk = e / TM; }
            const int gi = i0 + ii, gk = k0 + kk;
            float val = 0.f;
            if (gi < g.M && gk < g.K) {
                if constexpr (ALOAD == A_DIVERGENCE) val = div_at(g, gi, gk);
                else val = A[(long long)gi * g.sAi + (long long)gk * g.sAk];
            }
            As[kk][ii] = val;
        }
        // B tile: TK x TN
#pragma unroll
        for (int r = 0; r < 4; ++r) {
            const int e = t + r * NT;
            int kk, jj;
            if (g.sBj == 1) { jj = e % TN; kk = e / TN; }
            else { kk = e % TK; jj = e / TK; }
            const int gk = k0 + kk, gj = j0 + jj;
            Bs[kk][jj] = (gk < g.K && gj < g.N) ? B[(long long)gk * g.sBk + (long long)gj * g.sBj]
                                                : 0.f;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < TK; ++kk) {
            float av[4], bv[4];
#pragma unroll
            for (int r = 0; r < 4; ++r) av[r] = As[kk][ti + 16 * r];
#pragma unroll
            for (int c = 0; c < 4; ++c) bv[c] = Bs[kk][tj + 16 * c];
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[r][c] = fmaf(av[r], bv[c], acc[r][c]);
        }
        __syncthreads();
    }
    float* C = g.C + (long long)b * g.sCb;
#pragma unroll
    for (int r = 0; r < 4; ++r) {
        const int gi = i0 + ti + 16 * r;
        if (gi >= g.M) continue;
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int gj = j0 + tj + 16 * c;
            if (gj >= g.N) continue;
            float v = acc[r][c];
            if constexpr (EPI == EPI_SCALE) {
                v = v * g.scale;
            } else if constexpr (EPI == EPI_POISSON_REF || EPI == EPI_POISSON_ACC) {
                int kx, ky, kz;
                if (g.pz_layout == 1) { kx = gj; ky = gi; kz = 0; }
                else {
                    const long long gc = gj + g.col_off;
                    kx = (int)(gc % g.W);
                    ky = (int)(gc / g.W);
                    kz = gi;
                }
                v = v * 8.f;  // the forward transform's last-pass factor
                if (kx == 0 && ky == 0 && kz == 0) {
                    v = 0.f;
                } else if constexpr (EPI == EPI_POISSON_REF) {
                    // FP32 cosines combined in FP64 (solve_poisson_in_cosine_domain.cu:48-53)
                    v = v / poisson_den_ref(g.D > 1, g.fx0, g.fx1, g.fx2, g.cosk0, g.cosk1,
                                            g.cosk2, kx, ky, kz);
                } else {
                    float den = g.eig0[kx] + g.eig1[ky];
                    if (g.D > 1) den = den + g.eig2[kz];
                    v = v / den;
                }
            }
            C[(long long)gi * g.sCi + (long long)gj * g.sCj] = v;
        }
    }
}

template <int ALOAD, int EPI>
void launch_gemm(const GemmArgs& g, int batches, cudaStream_t st) {
    const dim3 grid(ceil_div(g.N, TN), ceil_div(g.M, TM), batches);
    gemm_kernel<ALOAD, EPI><<<grid, NT, 0, st>>>(g);
    TGV_CHECK_LAUNCH();
}

GemmArgs base_args(const DctPlan* p) {
    GemmArgs g{};
    g.W = p->W;
    g.H = p->H;
    g.D = p->D;
    g.scale = 1.f;
    g.cosk0 = p->cosk[0];
    g.cosk1 = p->cosk[1];
    g.cosk2 = p->cosk[2];
    g.eig0 = p->eig[0];
    g.eig1 = p->eig[1];
    g.eig2 = p->eig[2];
    return g;
}

// One separable pass along `axis` with matrix Mat (N x N row-major).
// planes > 0: the x and y passes run over that many planes instead of the plan's depth.
void pass(const DctPlan* p, int axis, const float* Mat, const float* in, float* out, int epi,
          float scale, int aload, const float* vx, const float* vy, const float* vz,
          cudaStream_t st, int planes = 0) {
    const long long W = p->W, H = p->H, D = planes > 0 ? planes : p->D, WH = W * H;
    GemmArgs g = base_args(p);
    g.scale = scale;
    g.vx = vx;
    g.vy = vy;
    g.vz = vz;
    int batches = 1;
    if (axis == 0) {
        // out[r][k] = sum_n in[r][n] Mat[k][n]
        g.M = (int)(H * D);
        g.N = (int)W;
        g.K = (int)W;
        g.A = in;
        g.sAi = W;
        g.sAk = 1;
        g.sAb = 0;
        g.B = Mat;
        g.sBk = 1;
        g.sBj = W;
        g.sBb = 0;
        g.C = out;
        g.sCi = W;
        g.sCj = 1;
        g.sCb = 0;
    } else if (axis == 1) {
        // out[z][k][x] = sum_n Mat[k][n] in[z][n][x]
        g.M = (int)H;
        g.N = (int)W;
        g.K = (int)H;
        g.A = Mat;
        g.sAi = H;
        g.sAk = 1;
        g.sAb = 0;
        g.B = in;
        g.sBk = W;
        g.sBj = 1;
        g.sBb = WH;
        g.C = out;
        g.sCi = W;
        g.sCj = 1;
        g.sCb = WH;
        batches = (int)D;
        g.pz_layout = 1;
    } else {
        g.M = (int)D;
        g.N = (int)WH;
        g.K = (int)D;
        g.A = Mat;
        g.sAi = D;
        g.sAk = 1;
        g.sAb = 0;
        g.B = in;
        g.sBk = WH;
        g.sBj = 1;
        g.sBb = 0;
        g.C = out;
        g.sCi = WH;
        g.sCj = 1;
        g.sCb = 0;
        g.pz_layout = 2;
    }
    g.fx0 = p->cosk_fx[0];
    g.fx1 = p->cosk_fx[1];
    g.fx2 = p->cosk_fx[2];
    if (aload == A_DIVERGENCE) {
        TGV_REQUIRE(axis == 0, "divergence fusion is on the x pass");
        launch_gemm<A_DIVERGENCE, EPI_NONE>(g, batches, st);
        return;
    }
    switch (epi) {
        case EPI_NONE: launch_gemm<A_PLAIN, EPI_NONE>(g, batches, st); break;
        case EPI_SCALE: launch_gemm<A_PLAIN, EPI_SCALE>(g, batches, st); break;
        case EPI_POISSON_REF: launch_gemm<A_PLAIN, EPI_POISSON_REF>(g, batches, st); break;
        case EPI_POISSON_ACC: launch_gemm<A_PLAIN, EPI_POISSON_ACC>(g, batches, st); break;
    }
}

// ---- element-wise kernels --------------------------------------------------------------
// One block row of threads per (y, z) row: x from the thread, no per-element divisions.
__global__ void divergence_kernel(const float* __restrict__ vx, const float* __restrict__ vy,
                                  const float* __restrict__ vz, int W, int H, int D,
                                  float* __restrict__ out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= W) return;
    const size_t WH = (size_t)W * H;
    const long long rows = (long long)H * D;
    for (long long row = blockIdx.y; row < rows; row += gridDim.y) {
        const int y = (int)(row % H), z = (int)(row / H);
        const size_t idx = (size_t)row * W + x;
        const float bx = (x > 0 ? vx[idx - 1] : 0.f) - vx[idx];
        const float by = (y > 0 ? vy[idx - W] : 0.f) - vy[idx];
        float s = bx + by;
        if (D > 1) s = s + ((z > 0 ? vz[idx - WH] : 0.f) - vz[idx]);
        out[idx] = s;
    }
}

// Transpose of the divergence above, per component: (B_a^T g)[j] = g[j + e_a] - g[j]
// below the last slice of axis a and -g[j] on it (B_a w = w[i - e_a] - w[i], and -w[i]
// on the first slice).  gz is written only when D > 1 (the 2-D divergence has no z term).
__global__ void divergence_transpose_kernel(const float* __restrict__ g, int W, int H, int D,
                                            float* __restrict__ gx, float* __restrict__ gy,
                                            float* __restrict__ gz) {
    const size_t n = (size_t)W * H * D, WH = (size_t)W * H;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(idx % W);
        const int y = (int)((idx / W) % H);
        const int z = (int)(idx / WH);
        const float gi = g[idx];
        gx[idx] = (x + 1 < W ? g[idx + 1] : 0.f) - gi;
        gy[idx] = (y + 1 < H ? g[idx + W] : 0.f) - gi;
        if (D > 1) gz[idx] = (z + 1 < D ? g[idx + WH] : 0.f) - gi;
    }
}

__global__ void poisson_kernel(const float* __restrict__ in, float* __restrict__ out, int W, int H,
                               int D, const float* cx, const float* cy, const float* cz,
                               const float* ex, const float* ey, const float* ez, int accurate) {
    const size_t n = (size_t)W * H * D;
    for (size_t idx = blockIdx.x * (size_t)blockDim.x + threadIdx.x; idx < n;
         idx += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(idx % W);
        const int y = (int)((idx / W) % H);
        const int z = (int)(idx / ((size_t)W * H));
        if (x == 0 && y == 0 && z == 0) {
            out[idx] = 0.f;
            continue;
        }
        if (accurate) {
            float den = ex[x] + ey[y];
            if (D > 1) den = den + ez[z];
            out[idx] = in[idx] / den;
        } else {
            double den = (D > 1 ? 6.0 : 4.0) - 2.0 * (double)cx[x] - 2.0 * (double)cy[y];
            if (D > 1) den -= 2.0 * (double)cz[z];
            out[idx] = (float)((double)in[idx] / den);
        }
    }
}

// mask_again: the masked processor multiplies r by the mask a second time when it
// does not add the background back (TGVDeshadeMaskedProcessor.cpp:203-211).
__global__ void epilogue_kernel(const float* __restrict__ u, float* __restrict__ l,
                                const float* __restrict__ mask, size_t n, int mask_shading,
                                int clamp, int add_back, int mask_again, float* __restrict__ r) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x) {
        const float ui = u[i];
        float li = l[i];
        float ri = ui - li;                       // TGVDeshadeProcessor.cpp:83
        if (mask) {
            const float m = mask[i];
            if (mask_shading) l[i] = li * m;      // :87
            ri = ri * m;                          // :88
        }
        if (clamp && ri < 0.f) ri = 0.f;         // :91-92
        if (add_back && mask) ri = ri + ui * (1.f - mask[i]);  // :275-279
        else if (mask_again && mask) ri = ri * mask[i];
        r[i] = ri;
    }
}

__global__ void log_kernel(float* x, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        x[i] = logf(x[i]);
}

__global__ void exp_kernel(float* x, size_t n) {
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n;
         i += (size_t)gridDim.x * blockDim.x)
        x[i] = expf(x[i]);
}

unsigned ew_grid(size_t n) {
    size_t b = (n + 255) / 256;
    if (b > 152 * 32) b = 152 * 32;
    return (unsigned)(b ? b : 1);
}

}  // namespace

size_t dct_plan_bytes(int W, int H, int D, size_t tmp_voxels) {
    size_t b = 0;
    const int N[3] = {W, H, D};
    for (int a = 0; a < 3; ++a)
        b += 2 * a256((size_t)N[a] * N[a] * 4) + 2 * a256((size_t)N[a] * 4) +
             a256((size_t)N[a] * 8);
    if (tmp_voxels == 0) tmp_voxels = (size_t)W * H * D;
    b += 2 * a256(tmp_voxels * 4) + 256;
    return b;
}

DctPlan* dct_plan_create(int W, int H, int D, size_t tmp_voxels) {
    DctPlan* p = new DctPlan();
    p->W = W;
    p->H = H;
    p->D = D;
    if (tmp_voxels == 0) tmp_voxels = (size_t)W * H * D;
    const size_t bytes = dct_plan_bytes(W, H, D, tmp_voxels);
    cudaError_t e = cudaMalloc(&p->block, bytes);
    if (e != cudaSuccess) {
        delete p;
        set_error(std::string("cudaMalloc of the DCT plan: ") + cudaGetErrorString(e));
        throw Error{TGVDCT_ERR_OOM};
    }
    char* c = (char*)p->block;
    const int N[3] = {W, H, D};
    for (int a = 0; a < 3; ++a) {
        const size_t n = (size_t)N[a];
        p->fwd[a] = (float*)c;
        c += a256(n * n * 4);
        p->inv[a] = (float*)c;
        c += a256(n * n * 4);
        p->cosk[a] = (float*)c;
        c += a256(n * 4);
        p->eig[a] = (float*)c;
        c += a256(n * 4);
        p->cosk_fx[a] = (long long*)c;
        c += a256(n * 8);
        std::vector<float> C(n * n), S(n * n), E(n);
        for (size_t k = 0; k < n; ++k) {
            for (size_t m = 0; m < n; ++m) {
                const double cv = cospi_host(((double)m + 0.5) * (double)k / (double)n);
                C[k * n + m] = (float)cv;                        // forward: row k, column m
                S[m * n + k] = (float)(k == 0 ? cv : 2.0 * cv);  // inverse: row m, column k
            }
            const double s = std::sin(3.14159265358979323846 * (double)k / (2.0 * (double)n));
            E[k] = (float)(4.0 * s * s);
        }
        try {
            TGV_CUDA(cudaMemcpy(p->fwd[a], C.data(), n * n * 4, cudaMemcpyHostToDevice));
            TGV_CUDA(cudaMemcpy(p->inv[a], S.data(), n * n * 4, cudaMemcpyHostToDevice));
            TGV_CUDA(cudaMemcpy(p->eig[a], E.data(), n * 4, cudaMemcpyHostToDevice));
            cosk_kernel<<<ceil_div(n, 128), 128>>>(p->cosk[a], (int)n);
            TGV_CHECK_LAUNCH();
        } catch (...) {
            cudaFree(p->block);
            delete p;
            throw;
        }
    }
    p->tmp[0] = (float*)c;
    c += a256(tmp_voxels * 4);
    p->tmp[1] = (float*)c;
    c += a256(tmp_voxels * 4);
    int* inexact = (int*)c;
    cudaError_t se = cudaMemset(inexact, 0, sizeof(int));
    const bool small = W <= 256 && H <= 256 && D <= 256;
    for (int a = 0; a < 3 && se == cudaSuccess && small; ++a) {
        cosk_fx_kernel<<<ceil_div((size_t)N[a], 128), 128>>>(p->cosk[a], N[a], p->cosk_fx[a],
                                                            inexact);
        se = cudaGetLastError();
    }
    // The synchronous copy waits for the set-up kernels before it (the same legacy
    // stream). No device-wide synchronisation: that is refused, and invalidates the
    // capture, while another thread captures a loop graph.
    int h_inexact = 1;
    if (se == cudaSuccess) se = cudaMemcpy(&h_inexact, inexact, sizeof(int), cudaMemcpyDeviceToHost);
    if (se != cudaSuccess) {
        cudaFree(p->block);
        delete p;
        set_error(std::string("DCT plan setup: ") + cudaGetErrorString(se));
        throw Error{TGVDCT_ERR_CUDA};
    }
    if (!small || h_inexact)  // the FP64 form of the reference eigenvalues
        for (int a = 0; a < 3; ++a) p->cosk_fx[a] = nullptr;
    return p;
}

void dct_plan_destroy(DctPlan* p) {
    if (!p) return;
    if (p->tc_block) cudaFree(p->tc_block);
    if (p->pipe_block) cudaFree(p->pipe_block);
    cudaFree(p->block);
    delete p;
}

void divergence(DctPlan* p, const float* vx, const float* vy, const float* vz, float* out,
                cudaStream_t st) {
    const long long rows = (long long)p->H * p->D;
    const dim3 grid(ceil_div((size_t)p->W, 128), (unsigned)std::min(rows, 65535ll));
    divergence_kernel<<<grid, 128, 0, st>>>(vx, vy, vz, p->W, p->H, p->D, out);
    TGV_CHECK_LAUNCH();
}

// A separable pass on the CUDA cores (FP32) or the tensor cores (dct_tc.cu).
void any_pass(DctPlan* p, int axis, bool inverse, const float* in, float* out, int epi, float scale,
              int dct_mode, cudaStream_t st) {
    if (dct_mode == TGVDCT_DCT_FP32) {
        pass(p, axis, inverse ? p->inv[axis] : p->fwd[axis], in, out, epi, scale, A_PLAIN, 0, 0, 0,
             st);
    } else if (!pass_pipe(p, axis, inverse, in, out, epi, scale, dct_mode, st)) {
        pass_tc(p, axis, inverse, in, out, epi, scale, false, nullptr, nullptr, nullptr, dct_mode,
                st);
    }
}

void check_mode(DctPlan* p, int dct_mode) {
    TGV_REQUIRE(dct_mode == TGVDCT_DCT_FP32 || dct_mode == TGVDCT_DCT_TF32 ||
                    dct_mode == TGVDCT_DCT_BF16X3,
                "unknown DCT mode");
    if (dct_mode != TGVDCT_DCT_FP32 && !dct_tc_supported(p)) {
        set_error("tensor-core DCT modes need every side <= 256");
        throw Error{TGVDCT_ERR_UNSUPPORTED};
    }
}

void cosine_transform(DctPlan* p, const float* in, float* out, int dct_mode, cudaStream_t st) {
    check_mode(p, dct_mode);
    if (p->D == 1) {
        any_pass(p, 0, false, in, p->tmp[0], EPI_NONE, 1.f, dct_mode, st);
        any_pass(p, 1, false, p->tmp[0], out, EPI_SCALE, 8.f, dct_mode, st);
    } else {
        any_pass(p, 0, false, in, p->tmp[0], EPI_NONE, 1.f, dct_mode, st);
        any_pass(p, 1, false, p->tmp[0], p->tmp[1], EPI_NONE, 1.f, dct_mode, st);
        any_pass(p, 2, false, p->tmp[1], out, EPI_SCALE, 8.f, dct_mode, st);
    }
}

void inverse_cosine_transform(DctPlan* p, const float* in, float* out, int dct_mode,
                              cudaStream_t st) {
    check_mode(p, dct_mode);
    const float s = (float)(1.0 / ((double)p->W * p->H * p->D * 8.0));
    if (p->D == 1) {
        any_pass(p, 0, true, in, p->tmp[0], EPI_NONE, 1.f, dct_mode, st);
        any_pass(p, 1, true, p->tmp[0], out, EPI_SCALE, s, dct_mode, st);
    } else {
        any_pass(p, 0, true, in, p->tmp[0], EPI_NONE, 1.f, dct_mode, st);
        any_pass(p, 1, true, p->tmp[0], p->tmp[1], EPI_NONE, 1.f, dct_mode, st);
        any_pass(p, 2, true, p->tmp[1], out, EPI_SCALE, s, dct_mode, st);
    }
}

void solve_poisson(DctPlan* p, const float* in, float* out, int eigen_mode, cudaStream_t st) {
    const size_t n = (size_t)p->W * p->H * p->D;
    poisson_kernel<<<ew_grid(n), 256, 0, st>>>(in, out, p->W, p->H, p->D, p->cosk[0], p->cosk[1],
                                               p->cosk[2], p->eig[0], p->eig[1], p->eig[2],
                                               eigen_mode == TGVDCT_EIGEN_ACCURATE ? 1 : 0);
    TGV_CHECK_LAUNCH();
}

void poisson_solve(DctPlan* p, const float* rhs, float* l, int dct_mode, int eigen_mode,
                   cudaStream_t st) {
    check_mode(p, dct_mode);
    const int epi = eigen_mode == TGVDCT_EIGEN_ACCURATE ? EPI_POISSON_ACC : EPI_POISSON_REF;
    const float s = (float)(1.0 / ((double)p->W * p->H * p->D * 8.0));
    float* t0 = p->tmp[0];
    float* t1 = p->tmp[1];
    any_pass(p, 0, false, rhs, t0, EPI_NONE, 1.f, dct_mode, st);
    if (p->D == 1) {
        any_pass(p, 1, false, t0, t1, epi, 1.f, dct_mode, st);
        any_pass(p, 0, true, t1, t0, EPI_NONE, 1.f, dct_mode, st);
        any_pass(p, 1, true, t0, l, EPI_SCALE, s, dct_mode, st);
    } else {
        // forward x, y, z (+ division); inverse z, y, x: the z contractions are adjacent,
        // so a z-slab decomposition needs one transposition to z pencils and one back
        any_pass(p, 1, false, t0, t1, EPI_NONE, 1.f, dct_mode, st);
        any_pass(p, 2, false, t1, t0, epi, 1.f, dct_mode, st);
        any_pass(p, 2, true, t0, t1, EPI_NONE, 1.f, dct_mode, st);
        any_pass(p, 1, true, t1, t0, EPI_NONE, 1.f, dct_mode, st);
        any_pass(p, 0, true, t0, l, EPI_SCALE, s, dct_mode, st);
    }
}

void poisson_integrate(DctPlan* p, const float* vx, const float* vy, const float* vz, float* l,
                       int dct_mode, int eigen_mode, cudaStream_t st) {
    NvtxRange range("tgvdct poisson integration");
    check_mode(p, dct_mode);
    const int epi = eigen_mode == TGVDCT_EIGEN_ACCURATE ? EPI_POISSON_ACC : EPI_POISSON_REF;
    const float s = (float)(1.0 / ((double)p->W * p->H * p->D * 8.0));
    float* t0 = p->tmp[0];
    float* t1 = p->tmp[1];
    // forward: x (divergence fused into the operand load), y, z (+ Poisson division)
    if (dct_mode == TGVDCT_DCT_FP32)
        pass(p, 0, p->fwd[0], nullptr, t0, EPI_NONE, 1.f, A_DIVERGENCE, vx, vy, vz, st);
    else if (dct_pipe_supported(p)) {
        // the pipelined passes take a plain operand: divergence first, into t1
        divergence(p, vx, vy, vz, t1, st);
        if (!pass_pipe(p, 0, false, t1, t0, EPI_NONE, 1.f, dct_mode, st))
            pass_tc(p, 0, false, nullptr, t0, EPI_NONE, 1.f, true, vx, vy, vz, dct_mode, st);
    } else
        pass_tc(p, 0, false, nullptr, t0, EPI_NONE, 1.f, true, vx, vy, vz, dct_mode, st);
    if (p->D == 1) {
        any_pass(p, 1, false, t0, t1, epi, 1.f, dct_mode, st);
        any_pass(p, 0, true, t1, t0, EPI_NONE, 1.f, dct_mode, st);
        any_pass(p, 1, true, t0, l, EPI_SCALE, s, dct_mode, st);
    } else {
        // forward x, y, z (+ division); inverse z, y, x: the z contractions are adjacent,
        // so a z-slab decomposition needs one transposition to z pencils and one back
        any_pass(p, 1, false, t0, t1, EPI_NONE, 1.f, dct_mode, st);
        any_pass(p, 2, false, t1, t0, epi, 1.f, dct_mode, st);
        any_pass(p, 2, true, t0, t1, EPI_NONE, 1.f, dct_mode, st);
        any_pass(p, 1, true, t1, t0, EPI_NONE, 1.f, dct_mode, st);
        any_pass(p, 0, true, t0, l, EPI_SCALE, s, dct_mode, st);
    }
}

// ---- z-slab decomposition of the Poisson integration (FP32 contractions) ---------
// The single-volume order is: divergence fused into the forward x pass, forward y,
// forward z with the division, inverse z, inverse y, inverse x (scaled).  A rank
// that holds z-planes runs the x and y passes on its planes, the z passes run on z
// pencils (all planes of a span of columns), and the inverse y and x passes run on
// the rank's planes again.  Each output value is the same dot product, accumulated
// in the same order, as in the single-volume solve, so the results agree bit for bit.

void slab_poisson_xy(DctPlan* p, const float* vx, const float* vy, const float* vz, float* out,
                     cudaStream_t st) {
    pass(p, 0, p->fwd[0], nullptr, p->tmp[0], EPI_NONE, 1.f, A_DIVERGENCE, vx, vy, vz, st);
    pass(p, 1, p->fwd[1], p->tmp[0], out, EPI_NONE, 1.f, A_PLAIN, 0, 0, 0, st);
}

void slab_poisson_inverse_yx(DctPlan* p, const float* in, float* out, int planes, float scale,
                             cudaStream_t st) {
    pass(p, 1, p->inv[1], in, p->tmp[0], EPI_NONE, 1.f, A_PLAIN, 0, 0, 0, st, planes);
    pass(p, 0, p->inv[0], p->tmp[0], out, EPI_SCALE, scale, A_PLAIN, 0, 0, 0, st, planes);
}

// in, out: D x columns (z-major), the columns [col_off, col_off + columns) of the
// W*H plane; forward z (x 8, the division by the Laplacian eigenvalues, DC = 0),
// then inverse z.  Uses tmp[0] (D x columns).
void pencil_poisson_z(DctPlan* p, const float* in, float* out, long long columns,
                      long long col_off, int eigen_mode, cudaStream_t st) {
    const int epi = eigen_mode == TGVDCT_EIGEN_ACCURATE ? EPI_POISSON_ACC : EPI_POISSON_REF;
    for (int step = 0; step < 2; ++step) {
        GemmArgs g = base_args(p);
        g.M = p->D;
        g.N = (int)columns;
        g.K = p->D;
        g.A = step == 0 ? p->fwd[2] : p->inv[2];
        g.sAi = p->D;
        g.sAk = 1;
        g.B = step == 0 ? in : p->tmp[0];
        g.sBk = columns;
        g.sBj = 1;
        g.C = step == 0 ? p->tmp[0] : out;
        g.sCi = columns;
        g.sCj = 1;
        g.pz_layout = 2;
        g.col_off = col_off;
        g.fx0 = p->cosk_fx[0];
        g.fx1 = p->cosk_fx[1];
        g.fx2 = p->cosk_fx[2];
        if (step == 1) launch_gemm<A_PLAIN, EPI_NONE>(g, 1, st);
        else if (epi == EPI_POISSON_ACC) launch_gemm<A_PLAIN, EPI_POISSON_ACC>(g, 1, st);
        else launch_gemm<A_PLAIN, EPI_POISSON_REF>(g, 1, st);
    }
}

void poisson_integrate_adjoint(DctPlan* p, const float* gl, float* scratch, float* gvx,
                               float* gvy, float* gvz, int dct_mode, int eigen_mode,
                               cudaStream_t st) {
    // l = M B v with M = S diag(1/eig) C symmetric (S = C^T W): the adjoint is B^T M g
    poisson_solve(p, gl, scratch, dct_mode, eigen_mode, st);
    const size_t n = (size_t)p->W * p->H * p->D;
    divergence_transpose_kernel<<<ew_grid(n), 256, 0, st>>>(scratch, p->W, p->H, p->D, gvx, gvy,
                                                             gvz);
    TGV_CHECK_LAUNCH();
}

void deshade_epilogue(const float* u, float* l, const float* mask, size_t n, bool mask_shading,
                      bool clamp, bool add_back, float* r, cudaStream_t st, bool mask_again) {
    epilogue_kernel<<<ew_grid(n), 256, 0, st>>>(u, l, mask, n, mask_shading ? 1 : 0,
                                                clamp ? 1 : 0, add_back ? 1 : 0,
                                                mask_again ? 1 : 0, r);
    TGV_CHECK_LAUNCH();
}

void log_inplace(float* x, size_t n, cudaStream_t st) {
    log_kernel<<<ew_grid(n), 256, 0, st>>>(x, n);
    TGV_CHECK_LAUNCH();
}

void exp_inplace(float* x, size_t n, cudaStream_t st) {
    exp_kernel<<<ew_grid(n), 256, 0, st>>>(x, n);
    TGV_CHECK_LAUNCH();
}

}  // namespace tgvdct

// Learned walker budgets: source features (K5) and a small FP32 MLP with
// hand-written forward, backward and Adam kernels (K6).  No reference
// counterpart: the reference runs every query with the same walker count.
//
// Network: x[8] -> (x - mu) / sigma -> z1 = W1^T x + b1 [64] -> relu ->
//          z2 = W2^T a1 + b2 [64] -> relu -> y = w3 . a2 + b3.
// Loss: mean squared error against normalised targets.  Parameters live in
// one flat FP32 array:
//   W1[8][64] @0, b1[64] @512, W2[64][64] @576, b2[64] @4672, w3[64] @4736, b3 @4800.
// Every reduction runs in a fixed order (one thread per parameter looping
// over the batch), so gradients are deterministic and comparable with the
// FP64 reference in the tests.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "ptw_internal.cuh"

struct ptw_mlp {
    float *params = nullptr, *grad = nullptr, *m = nullptr, *v = nullptr;  // [PTW_MLP_NPARAMS]
    float norm[2 * PTW_MLP_IN + 2];  // mu[8], sigma[8], t_mu, t_sigma (host)
    uint64_t step = 0;
    int device = 0;
    cudaStream_t stream = nullptr;
};

namespace ptw {
namespace {

constexpr int IN = PTW_MLP_IN, H = PTW_MLP_HIDDEN;
constexpr int OW1 = 0, OB1 = IN * H, OW2 = OB1 + H, OB2 = OW2 + H * H, OW3 = OB2 + H, OB3 = OW3 + H;
static_assert(OB3 + 1 == PTW_MLP_NPARAMS, "parameter layout");

struct Norm {
    float mu[IN], sd[IN], tmu, tsd;
};

// One thread per sample: z1, z2 (pre-activations) and y.
__global__ void k_mlp_fwd(const float *__restrict__ P, Norm nm, const float *__restrict__ x, uint32_t B,
                          float *z1, float *z2, float *y)
{
    __shared__ float s[PTW_MLP_NPARAMS];
    for (int i = threadIdx.x; i < PTW_MLP_NPARAMS; i += blockDim.x) s[i] = P[i];
    __syncthreads();
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    float xi[IN];
#pragma unroll
    for (int k = 0; k < IN; ++k) xi[k] = (x[(uint64_t)b * IN + k] - nm.mu[k]) / nm.sd[k];
    float a1[H];
    for (int i = 0; i < H; ++i) {
        float acc = s[OB1 + i];
#pragma unroll
        for (int k = 0; k < IN; ++k) acc = fmaf(xi[k], s[OW1 + k * H + i], acc);
        z1[(uint64_t)b * H + i] = acc;
        a1[i] = acc > 0.f ? acc : 0.f;
    }
    float out = s[OB3];
    for (int j = 0; j < H; ++j) {
        float acc = s[OB2 + j];
        for (int i = 0; i < H; ++i) acc = fmaf(a1[i], s[OW2 + i * H + j], acc);
        z2[(uint64_t)b * H + j] = acc;
        out = fmaf(acc > 0.f ? acc : 0.f, s[OW3 + j], out);
    }
    y[b] = out;
}

// One thread per sample: e = dL/dy, dz2, dz1.
__global__ void k_mlp_bwd(const float *__restrict__ P, Norm nm, const float *__restrict__ t, uint32_t B,
                          const float *z1, const float *z2, const float *y, float *e, float *dz1, float *dz2,
                          float *loss_terms)
{
    __shared__ float s[PTW_MLP_NPARAMS];
    for (int i = threadIdx.x; i < PTW_MLP_NPARAMS; i += blockDim.x) s[i] = P[i];
    __syncthreads();
    const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= B) return;
    const float tn = (t[b] - nm.tmu) / nm.tsd;
    const float d = y[b] - tn;
    loss_terms[b] = d * d;
    const float eb = 2.f * d / (float)B;
    e[b] = eb;
    float g2[H];
    for (int j = 0; j < H; ++j) {
        g2[j] = z2[(uint64_t)b * H + j] > 0.f ? eb * s[OW3 + j] : 0.f;
        dz2[(uint64_t)b * H + j] = g2[j];
    }
    for (int i = 0; i < H; ++i) {
        float acc = 0.f;
        if (z1[(uint64_t)b * H + i] > 0.f)
            for (int j = 0; j < H; ++j) acc = fmaf(g2[j], s[OW2 + i * H + j], acc);
        dz1[(uint64_t)b * H + i] = acc;
    }
}

// One thread per parameter, summing over the batch in order.
__global__ void k_mlp_grad(Norm nm, const float *__restrict__ x, uint32_t B, const float *z1, const float *z2,
                           const float *e, const float *dz1, const float *dz2, float *G)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= PTW_MLP_NPARAMS) return;
    float acc = 0.f;
    if (p < OB1) {
        const int k = p / H, i = p % H;
        for (uint32_t b = 0; b < B; ++b)
            acc = fmaf((x[(uint64_t)b * IN + k] - nm.mu[k]) / nm.sd[k], dz1[(uint64_t)b * H + i], acc);
    } else if (p < OW2) {
        const int i = p - OB1;
        for (uint32_t b = 0; b < B; ++b) acc += dz1[(uint64_t)b * H + i];
    } else if (p < OB2) {
        const int i = (p - OW2) / H, j = (p - OW2) % H;
        for (uint32_t b = 0; b < B; ++b) {
            const float a = z1[(uint64_t)b * H + i];
            if (a > 0.f) acc = fmaf(a, dz2[(uint64_t)b * H + j], acc);
        }
    } else if (p < OW3) {
        const int j = p - OB2;
        for (uint32_t b = 0; b < B; ++b) acc += dz2[(uint64_t)b * H + j];
    } else if (p < OB3) {
        const int j = p - OW3;
        for (uint32_t b = 0; b < B; ++b) {
            const float a = z2[(uint64_t)b * H + j];
            if (a > 0.f) acc = fmaf(e[b], a, acc);
        }
    } else {
        for (uint32_t b = 0; b < B; ++b) acc += e[b];
    }
    G[p] = acc;
}

__global__ void k_adam(float *P, const float *G, float *M, float *V, float lr, float b1, float b2, float eps,
                       float c1, float c2)
{
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= PTW_MLP_NPARAMS) return;
    const float g = G[p];
    const float m = b1 * M[p] + (1.f - b1) * g;
    const float v = b2 * V[p] + (1.f - b2) * g * g;
    M[p] = m;
    V[p] = v;
    P[p] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
}

__global__ void k_gather_rows(const float *src, const uint32_t *idx, uint32_t B, int w, float *dst)
{
    const uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= (uint64_t)B * w) return;
    const uint64_t b = i / w;
    dst[i] = src[(uint64_t)idx[b] * w + (i - b * w)];
}

// ---- K5: source features, one warp per source -----------------------------
//  f0 log(1+deg)          f1 mean log(1+deg(u))    f2 max log(1+deg(u))
//  f3 min log(1+deg(u))   f4 log(1+sum deg(u))     f5 std log(1+deg(u))
//  f6 fraction of neighbours of degree 1          f7 log(1+sum deg(u)/deg)
__global__ void k_features(const uint2 *adj, const uint32_t *col, const uint32_t *src, uint32_t ns, float *f)
{
    const uint32_t lane = threadIdx.x & 31;
    const uint64_t warps = ((uint64_t)gridDim.x * blockDim.x) >> 5;
    for (uint64_t q = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) >> 5; q < ns; q += warps) {
        const uint2 a = adj[src[q]];
        double s1 = 0, s2 = 0, sdeg = 0;
        float mx = -1e30f, mn = 1e30f;
        uint32_t ones = 0;
        for (uint32_t r = lane; r < a.y; r += 32) {
            const uint32_t du = adj[col[a.x + r]].y;
            const double l = log1p((double)du);
            s1 += l;
            s2 += l * l;
            sdeg += du;
            mx = fmaxf(mx, (float)l);
            mn = fminf(mn, (float)l);
            ones += du == 1;
        }
        for (int o = 16; o; o >>= 1) {
            s1 += __shfl_xor_sync(0xffffffffu, s1, o);
            s2 += __shfl_xor_sync(0xffffffffu, s2, o);
            sdeg += __shfl_xor_sync(0xffffffffu, sdeg, o);
            mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
            mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
            ones += __shfl_xor_sync(0xffffffffu, ones, o);
        }
        if (lane == 0) {
            const double d = a.y ? (double)a.y : 1.0;
            const double mean = a.y ? s1 / d : 0.0;
            const double var = a.y ? fmax(s2 / d - mean * mean, 0.0) : 0.0;
            float *o = f + q * IN;
            o[0] = (float)log1p((double)a.y);
            o[1] = (float)mean;
            o[2] = a.y ? mx : 0.f;
            o[3] = a.y ? mn : 0.f;
            o[4] = (float)log1p(sdeg);
            o[5] = (float)sqrt(var);
            o[6] = a.y ? (float)(ones / d) : 0.f;
            o[7] = (float)log1p(sdeg / d);
        }
    }
}

Norm host_norm(const ptw_mlp *m)
{
    Norm n;
    for (int k = 0; k < IN; ++k) {
        n.mu[k] = m->norm[k];
        n.sd[k] = m->norm[IN + k] > 0 ? m->norm[IN + k] : 1.f;
    }
    n.tmu = m->norm[2 * IN];
    n.tsd = m->norm[2 * IN + 1] > 0 ? m->norm[2 * IN + 1] : 1.f;
    return n;
}

struct MlpScratch {
    float *x = nullptr, *t = nullptr, *z1 = nullptr, *z2 = nullptr, *y = nullptr, *e = nullptr, *dz1 = nullptr,
          *dz2 = nullptr, *lt = nullptr;
    cudaStream_t st;
    explicit MlpScratch(cudaStream_t s) : st(s) {}
    cudaError_t alloc(uint32_t B)
    {
        cudaError_t r = cudaSuccess;
        auto a = [&](float **p, uint64_t n) {
            if (r == cudaSuccess) r = cudaMallocAsync((void **)p, std::max<uint64_t>(n, 1) * 4, st);
        };
        a(&x, (uint64_t)B * IN);
        a(&t, B);
        a(&z1, (uint64_t)B * H);
        a(&z2, (uint64_t)B * H);
        a(&y, B);
        a(&e, B);
        a(&dz1, (uint64_t)B * H);
        a(&dz2, (uint64_t)B * H);
        a(&lt, B);
        return r;
    }
    ~MlpScratch()
    {
        for (float *p : {x, t, z1, z2, y, e, dz1, dz2, lt})
            if (p) cudaFreeAsync(p, st);
    }
};

// Loss and gradient of one batch already in s.x / s.t; grad in m->grad.
int batch_grad(ptw_mlp *m, MlpScratch &s, uint32_t B, double *loss)
{
    const Norm nm = host_norm(m);
    const unsigned g = (B + 127) / 128;
    k_mlp_fwd<<<g, 128, 0, m->stream>>>(m->params, nm, s.x, B, s.z1, s.z2, s.y);
    k_mlp_bwd<<<g, 128, 0, m->stream>>>(m->params, nm, s.t, B, s.z1, s.z2, s.y, s.e, s.dz1, s.dz2, s.lt);
    k_mlp_grad<<<(PTW_MLP_NPARAMS + 127) / 128, 128, 0, m->stream>>>(nm, s.x, B, s.z1, s.z2, s.e, s.dz1, s.dz2,
                                                                     m->grad);
    PTW_CUDA(cudaGetLastError());
    if (loss) {
        std::vector<float> lt(B);
        PTW_CUDA(cudaMemcpyAsync(lt.data(), s.lt, B * 4ull, cudaMemcpyDeviceToHost, m->stream));
        PTW_CUDA(cudaStreamSynchronize(m->stream));
        double acc = 0;
        for (float v : lt) acc += v;
        *loss = acc / B;
    }
    return PTW_OK;
}

}  // namespace
}  // namespace ptw

using namespace ptw;

extern "C" int ptw_source_features(ptw_graph *g, const uint32_t *h_sources, uint32_t ns, float *h_feat)
try {
    if (!g || (ns && (!h_sources || !h_feat))) return fail(PTW_EINVAL, "null argument");
    if (!ns) return PTW_OK;
    PTW_CUDA(cudaSetDevice(g->device));
    const uint32_t n = g->dg.n;
    std::vector<uint32_t> ids(ns);
    for (uint32_t i = 0; i < ns; ++i) {
        const uint32_t *p = std::lower_bound(g->h_names, g->h_names + n, h_sources[i]);
        if (p == g->h_names + n || *p != h_sources[i])
            return fail(PTW_EINVAL, "source " + std::to_string(h_sources[i]) + " is not a vertex of the graph");
        ids[i] = g->h_idx2int[p - g->h_names];
    }
    cudaStream_t st = g->stream;
    uint32_t *d_src = nullptr;
    float *d_f = nullptr;
    PTW_CUDA(cudaMallocAsync(&d_src, ns * 4ull, st));
    cudaError_t e = cudaMallocAsync(&d_f, ns * 4ull * IN, st);
    if (e != cudaSuccess) {
        cudaFreeAsync(d_src, st);
        return cuda_fail(e, "feature buffer");
    }
    e = cudaMemcpyAsync(d_src, ids.data(), ns * 4ull, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        const unsigned grid = (unsigned)std::min<uint64_t>(((uint64_t)ns * 32 + 255) / 256, 65535);
        k_features<<<std::max(grid, 1u), 256, 0, st>>>(g->dg.adj, g->dg.col, d_src, ns, d_f);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(h_feat, d_f, ns * 4ull * IN, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFreeAsync(d_src, st);
    cudaFreeAsync(d_f, st);
    if (e != cudaSuccess) return cuda_fail(e, "source features");
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_mlp_create(uint64_t seed, ptw_mlp **out)
try {
    if (!out) return fail(PTW_EINVAL, "null argument");
    *out = nullptr;
    ptw_mlp *m = new (std::nothrow) ptw_mlp();
    if (!m) return fail(PTW_ENOMEM, "host allocation failed");
    std::memset(m->norm, 0, sizeof(m->norm));
    for (int k = 0; k < IN; ++k) m->norm[IN + k] = 1.f;
    m->norm[2 * IN + 1] = 1.f;
    int rc = PTW_OK;
    cudaError_t e = cudaGetDevice(&m->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking);
    for (float **p : {&m->params, &m->grad, &m->m, &m->v})
        if (e == cudaSuccess) e = device_malloc((void **)p, PTW_MLP_NPARAMS * 4);
    if (e != cudaSuccess) {
        rc = cuda_fail(e, "MLP allocation");
    } else {
        // He-uniform initialisation from a 64-bit LCG (Knuth MMIX constants);
        // biases zero.
        std::vector<float> h(PTW_MLP_NPARAMS, 0.f);
        uint64_t st = seed * 6364136223846793005ull + 1442695040888963407ull;
        auto uni = [&]() {
            st = st * 6364136223846793005ull + 1442695040888963407ull;
            return (double)(st >> 11) / 9007199254740992.0 * 2.0 - 1.0;
        };
        for (int i = OW1; i < OB1; ++i) h[i] = (float)(uni() * std::sqrt(6.0 / IN));
        for (int i = OW2; i < OB2; ++i) h[i] = (float)(uni() * std::sqrt(6.0 / H));
        for (int i = OW3; i < OB3; ++i) h[i] = (float)(uni() * std::sqrt(3.0 / H));
        e = cudaMemcpy(m->params, h.data(), PTW_MLP_NPARAMS * 4, cudaMemcpyHostToDevice);
        if (e == cudaSuccess) e = cudaMemset(m->m, 0, PTW_MLP_NPARAMS * 4);
        if (e == cudaSuccess) e = cudaMemset(m->v, 0, PTW_MLP_NPARAMS * 4);
        if (e != cudaSuccess) rc = cuda_fail(e, "MLP init");
    }
    if (rc != PTW_OK) {
        ptw_mlp_free(m);
        return rc;
    }
    *out = m;
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_mlp_set_params(ptw_mlp *m, const float *h_params, const float *h_norm)
try {
    if (!m) return fail(PTW_EINVAL, "null model");
    PTW_CUDA(cudaSetDevice(m->device));
    if (h_params) PTW_CUDA(cudaMemcpy(m->params, h_params, PTW_MLP_NPARAMS * 4, cudaMemcpyHostToDevice));
    if (h_norm) std::memcpy(m->norm, h_norm, sizeof(m->norm));
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_mlp_get_params(const ptw_mlp *m, float *h_params, float *h_norm)
try {
    if (!m) return fail(PTW_EINVAL, "null model");
    PTW_CUDA(cudaSetDevice(m->device));
    if (h_params) PTW_CUDA(cudaMemcpy(h_params, m->params, PTW_MLP_NPARAMS * 4, cudaMemcpyDeviceToHost));
    if (h_norm) std::memcpy(h_norm, m->norm, sizeof(m->norm));
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_mlp_forward(ptw_mlp *m, const float *h_x, uint32_t B, float *h_y)
try {
    if (!m || (B && (!h_x || !h_y))) return fail(PTW_EINVAL, "null argument");
    if (!B) return PTW_OK;
    PTW_CUDA(cudaSetDevice(m->device));
    MlpScratch s(m->stream);
    PTW_CUDA(s.alloc(B));
    PTW_CUDA(cudaMemcpyAsync(s.x, h_x, (uint64_t)B * IN * 4, cudaMemcpyHostToDevice, m->stream));
    const Norm nm = host_norm(m);
    k_mlp_fwd<<<(B + 127) / 128, 128, 0, m->stream>>>(m->params, nm, s.x, B, s.z1, s.z2, s.y);
    PTW_CUDA(cudaGetLastError());
    std::vector<float> y(B);
    PTW_CUDA(cudaMemcpyAsync(y.data(), s.y, B * 4ull, cudaMemcpyDeviceToHost, m->stream));
    PTW_CUDA(cudaStreamSynchronize(m->stream));
    for (uint32_t b = 0; b < B; ++b) h_y[b] = y[b] * nm.tsd + nm.tmu;  // de-normalised prediction
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_mlp_grad(ptw_mlp *m, const float *h_x, const float *h_t, uint32_t B, double *h_loss,
                            float *h_grad)
try {
    if (!m || !B || !h_x || !h_t) return fail(PTW_EINVAL, "null argument or empty batch");
    PTW_CUDA(cudaSetDevice(m->device));
    MlpScratch s(m->stream);
    PTW_CUDA(s.alloc(B));
    PTW_CUDA(cudaMemcpyAsync(s.x, h_x, (uint64_t)B * IN * 4, cudaMemcpyHostToDevice, m->stream));
    PTW_CUDA(cudaMemcpyAsync(s.t, h_t, B * 4ull, cudaMemcpyHostToDevice, m->stream));
    int rc = batch_grad(m, s, B, h_loss);
    if (rc) return rc;
    if (h_grad) PTW_CUDA(cudaMemcpyAsync(h_grad, m->grad, PTW_MLP_NPARAMS * 4, cudaMemcpyDeviceToHost, m->stream));
    PTW_CUDA(cudaStreamSynchronize(m->stream));
    return PTW_OK;
} catch (...) {
    return host_exception();
}

extern "C" int ptw_mlp_train(ptw_mlp *m, const float *h_x, const float *h_t, uint32_t N, uint32_t batch,
                             uint32_t epochs, float lr, uint64_t seed, float *h_loss_curve)
try {
    if (!m || !N || !h_x || !h_t || !batch) return fail(PTW_EINVAL, "null argument or empty data");
    PTW_CUDA(cudaSetDevice(m->device));
    // Normalisation from the training data (features and target).
    for (int k = 0; k < IN; ++k) {
        double s = 0, s2 = 0;
        for (uint32_t i = 0; i < N; ++i) {
            s += h_x[(uint64_t)i * IN + k];
            s2 += (double)h_x[(uint64_t)i * IN + k] * h_x[(uint64_t)i * IN + k];
        }
        const double mu = s / N, var = std::max(s2 / N - mu * mu, 1e-12);
        m->norm[k] = (float)mu;
        m->norm[IN + k] = (float)std::sqrt(var);
    }
    {
        double s = 0, s2 = 0;
        for (uint32_t i = 0; i < N; ++i) {
            s += h_t[i];
            s2 += (double)h_t[i] * h_t[i];
        }
        const double mu = s / N, var = std::max(s2 / N - mu * mu, 1e-12);
        m->norm[2 * IN] = (float)mu;
        m->norm[2 * IN + 1] = (float)std::sqrt(var);
    }
    batch = std::min(batch, N);
    cudaStream_t st = m->stream;
    float *d_X = nullptr, *d_T = nullptr;
    uint32_t *d_idx = nullptr;
    PTW_CUDA(cudaMallocAsync(&d_X, (uint64_t)N * IN * 4, st));
    PTW_CUDA(cudaMallocAsync(&d_T, N * 4ull, st));
    PTW_CUDA(cudaMallocAsync(&d_idx, N * 4ull, st));
    MlpScratch s(st);
    int rc = PTW_OK;
    cudaError_t e = s.alloc(batch);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_X, h_x, (uint64_t)N * IN * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d_T, h_t, N * 4ull, cudaMemcpyHostToDevice, st);
    if (e != cudaSuccess) rc = cuda_fail(e, "training data upload");
    std::vector<uint32_t> perm(N);
    for (uint32_t i = 0; i < N; ++i) perm[i] = i;
    uint64_t rs = seed * 0x9E3779B97F4A7C15ull + 1;
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (uint32_t ep = 0; ep < epochs && rc == PTW_OK; ++ep) {
        for (uint32_t i = N - 1; i > 0; --i) {  // Fisher-Yates with an LCG
            rs = rs * 6364136223846793005ull + 1442695040888963407ull;
            std::swap(perm[i], perm[(rs >> 33) % (i + 1)]);
        }
        e = cudaMemcpyAsync(d_idx, perm.data(), N * 4ull, cudaMemcpyHostToDevice, st);
        if (e != cudaSuccess) {
            rc = cuda_fail(e, "permutation upload");
            break;
        }
        double ep_loss = 0;
        uint32_t nb = 0;
        for (uint32_t b0 = 0; b0 < N && rc == PTW_OK; b0 += batch) {
            const uint32_t B = std::min(batch, N - b0);
            k_gather_rows<<<(unsigned)(((uint64_t)B * IN + 255) / 256), 256, 0, st>>>(d_X, d_idx + b0, B, IN, s.x);
            k_gather_rows<<<(B + 255) / 256, 256, 0, st>>>(d_T, d_idx + b0, B, 1, s.t);
            double loss = 0;
            rc = batch_grad(m, s, B, h_loss_curve ? &loss : nullptr);
            if (rc) break;
            ++m->step;
            const float c1 = 1.f - std::pow(b1, (float)m->step), c2 = 1.f - std::pow(b2, (float)m->step);
            k_adam<<<(PTW_MLP_NPARAMS + 127) / 128, 128, 0, st>>>(m->params, m->grad, m->m, m->v, lr, b1, b2, eps,
                                                                  c1, c2);
            e = cudaGetLastError();
            if (e != cudaSuccess) rc = cuda_fail(e, "adam");
            ep_loss += loss;
            ++nb;
        }
        if (h_loss_curve) h_loss_curve[ep] = (float)(ep_loss / std::max(nb, 1u));
    }
    cudaFreeAsync(d_X, st);
    cudaFreeAsync(d_T, st);
    cudaFreeAsync(d_idx, st);
    if (rc == PTW_OK) PTW_CUDA(cudaStreamSynchronize(st));
    return rc;
} catch (...) {
    return host_exception();
}

extern "C" void ptw_mlp_free(ptw_mlp *m)
try {
    if (!m) return;
    cudaSetDevice(m->device);
    if (m->stream) cudaStreamSynchronize(m->stream);
    cudaFree(m->params);
    cudaFree(m->grad);
    cudaFree(m->m);
    cudaFree(m->v);
    if (m->stream) cudaStreamDestroy(m->stream);
    delete m;
} catch (...) {
    host_exception();
}

// mlp.cu -- the learned task-cost model: a small MLP (nin -> H -> H -> 1, ReLU, FP32 weights)
// trained on the device by hand-written kernels (forward, backward, Adam).
//
// Layout: row-major activations, X (B x nin), W1 (nin x H), W2 (H x H), W3 (H x 1);
// parameters live in one FP32 vector [W1 | b1 | W2 | b2 | W3 | b3] so that gradients and the
// optimizer state are vectors of the same shape.  Loss: mean squared error on log-time.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "host_state.hpp"

namespace palial {
namespace mlpk {

// C (M x N) = alpha * op(A) op(B) + beta * C, row-major; op(A) is M x K (TA: A stored K x M),
// op(B) is K x N (TB: B stored N x K).  16 x 16 tiles in shared memory.
template <bool TA, bool TB>
__global__ void gemm_kernel(int M, int N, int K, float alpha, const float *A, const float *B, float beta, float *C) {
    __shared__ float As[16][17], Bs[16][17];
    const int r = blockIdx.y * 16 + threadIdx.y, c = blockIdx.x * 16 + threadIdx.x;
    float acc = 0.f;
    for (int k0 = 0; k0 < K; k0 += 16) {
        const int ka = k0 + threadIdx.x, kb = k0 + threadIdx.y;
        // op(A)(r, ka): TA ? A[ka * M + r] : A[r * K + ka]
        As[threadIdx.y][threadIdx.x] = (r < M && ka < K) ? (TA ? A[(size_t)ka * M + r] : A[(size_t)r * K + ka]) : 0.f;
        // op(B)(kb, c): TB ? B[c * K + kb] : B[kb * N + c]
        Bs[threadIdx.y][threadIdx.x] = (kb < K && c < N) ? (TB ? B[(size_t)c * K + kb] : B[(size_t)kb * N + c]) : 0.f;
        __syncthreads();
#pragma unroll
        for (int q = 0; q < 16; q++) acc = fmaf(As[threadIdx.y][q], Bs[q][threadIdx.x], acc);
        __syncthreads();
    }
    if (r < M && c < N) {
        float *o = C + (size_t)r * N + c;
        *o = alpha * acc + (beta == 0.f ? 0.f : beta * *o);
    }
}

// Z (B x H) += bias, then optionally ReLU (in place)
__global__ void bias_act_kernel(float *Z, const float *b, int Bn, int H, int relu) {
    const long long total = (long long)Bn * H;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x) {
        float v = Z[e] + b[e % H];
        Z[e] = relu ? fmaxf(v, 0.f) : v;
    }
}

// dY = 2 (Y - T) / B ; loss partial sums
__global__ void loss_grad_kernel(const float *Y, const float *T, float *dY, int Bn, float *loss) {
    float s = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < Bn; i += gridDim.x * blockDim.x) {
        const float d = Y[i] - T[i];
        dY[i] = 2.f * d / (float)Bn;
        s += d * d;
    }
    for (int o = 16; o; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(loss, s / (float)Bn);
}

// dZ *= (A > 0) (ReLU derivative through the stored activation)
__global__ void relu_back_kernel(float *dZ, const float *A, long long total) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total; e += (long long)gridDim.x * blockDim.x)
        if (A[e] <= 0.f) dZ[e] = 0.f;
}

// db[j] = sum_i dZ[i, j]
__global__ void colsum_kernel(const float *dZ, int Bn, int H, float *db) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= H) return;
    float s = 0.f;
    for (int i = 0; i < Bn; i++) s += dZ[(size_t)i * H + j];
    db[j] = s;
}

__global__ void adam_kernel(float *p, const float *g, float *m, float *v, int n, float lr, float b1, float b2, float eps,
                            float bc1, float bc2) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        p[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    }
}

}  // namespace mlpk

namespace {
struct Mlp {
    int nin = 0, H = 0;
    size_t nparam = 0;
    DevBuf params, grads, m, v, X, T, H1, H2, Y, dY, dH1, dH2, loss;
    int step = 0;
    bool ready = false;
    size_t off_W1() const { return 0; }
    size_t off_b1() const { return (size_t)nin * H; }
    size_t off_W2() const { return off_b1() + H; }
    size_t off_b2() const { return off_W2() + (size_t)H * H; }
    size_t off_W3() const { return off_b2() + H; }
    size_t off_b3() const { return off_W3() + H; }
};
Mlp net;

template <bool TA, bool TB>
void gemm(int M, int N, int K, float alpha, const float *A, const float *B, float beta, float *C) {
    dim3 block(16, 16), grid((N + 15) / 16, (M + 15) / 16);
    note_launch();
    mlpk::gemm_kernel<TA, TB><<<grid, block>>>(M, N, K, alpha, A, B, beta, C);
}

int ensure_batch(int Bn) {
    palial_status *st = nullptr;
    const size_t b = (size_t)Bn;
    PALIAL_CK(net.X.ensure(sizeof(float) * b * net.nin), "alloc");
    PALIAL_CK(net.T.ensure(sizeof(float) * b), "alloc");
    PALIAL_CK(net.H1.ensure(sizeof(float) * b * net.H), "alloc");
    PALIAL_CK(net.H2.ensure(sizeof(float) * b * net.H), "alloc");
    PALIAL_CK(net.Y.ensure(sizeof(float) * b), "alloc");
    PALIAL_CK(net.dY.ensure(sizeof(float) * b), "alloc");
    PALIAL_CK(net.dH1.ensure(sizeof(float) * b * net.H), "alloc");
    PALIAL_CK(net.dH2.ensure(sizeof(float) * b * net.H), "alloc");
    PALIAL_CK(net.loss.ensure(sizeof(float) * 4), "alloc");
    return PALIAL_OK;
}

void forward(int Bn) {
    float *p = net.params.as<float>();
    const int H = net.H;
    gemm<false, false>(Bn, H, net.nin, 1.f, net.X.as<float>(), p + net.off_W1(), 0.f, net.H1.as<float>());
    note_launch();
    mlpk::bias_act_kernel<<<256, 256>>>(net.H1.as<float>(), p + net.off_b1(), Bn, H, 1);
    gemm<false, false>(Bn, H, H, 1.f, net.H1.as<float>(), p + net.off_W2(), 0.f, net.H2.as<float>());
    note_launch();
    mlpk::bias_act_kernel<<<256, 256>>>(net.H2.as<float>(), p + net.off_b2(), Bn, H, 1);
    gemm<false, false>(Bn, 1, H, 1.f, net.H2.as<float>(), p + net.off_W3(), 0.f, net.Y.as<float>());
    note_launch();
    mlpk::bias_act_kernel<<<64, 256>>>(net.Y.as<float>(), p + net.off_b3(), Bn, 1, 0);
}

// gradients of the mean squared error into net.grads; returns via net.loss[0]
void backward(int Bn) {
    float *p = net.params.as<float>(), *g = net.grads.as<float>();
    const int H = net.H;
    cudaMemsetAsync(net.loss.ptr, 0, sizeof(float));
    note_launch();
    mlpk::loss_grad_kernel<<<64, 256>>>(net.Y.as<float>(), net.T.as<float>(), net.dY.as<float>(), Bn,
                                        net.loss.as<float>());
    // layer 3: dW3 = H2^T dY, db3 = sum dY, dH2 = dY W3^T
    gemm<true, false>(H, 1, Bn, 1.f, net.H2.as<float>(), net.dY.as<float>(), 0.f, g + net.off_W3());
    note_launch();
    mlpk::colsum_kernel<<<1, 32>>>(net.dY.as<float>(), Bn, 1, g + net.off_b3());
    gemm<false, true>(Bn, H, 1, 1.f, net.dY.as<float>(), p + net.off_W3(), 0.f, net.dH2.as<float>());
    note_launch();
    mlpk::relu_back_kernel<<<256, 256>>>(net.dH2.as<float>(), net.H2.as<float>(), (long long)Bn * H);
    // layer 2
    gemm<true, false>(H, H, Bn, 1.f, net.H1.as<float>(), net.dH2.as<float>(), 0.f, g + net.off_W2());
    note_launch();
    mlpk::colsum_kernel<<<(H + 63) / 64, 64>>>(net.dH2.as<float>(), Bn, H, g + net.off_b2());
    gemm<false, true>(Bn, H, H, 1.f, net.dH2.as<float>(), p + net.off_W2(), 0.f, net.dH1.as<float>());
    note_launch();
    mlpk::relu_back_kernel<<<256, 256>>>(net.dH1.as<float>(), net.H1.as<float>(), (long long)Bn * H);
    // layer 1
    gemm<true, false>(net.nin, H, Bn, 1.f, net.X.as<float>(), net.dH1.as<float>(), 0.f, g + net.off_W1());
    note_launch();
    mlpk::colsum_kernel<<<(H + 63) / 64, 64>>>(net.dH1.as<float>(), Bn, H, g + net.off_b1());
}
}  // namespace
}  // namespace palial

using namespace palial;

extern "C" {

int palial_mlp_init(int nin, int hidden, uint64_t seed) {
    palial_status *st = nullptr;
    int rc = ensure_init(nullptr);
    if (rc) return rc;
    if (nin <= 0 || hidden <= 0 || hidden > 1024) return PALIAL_ERR_ARG;
    net = Mlp();
    net.nin = nin;
    net.H = hidden;
    net.nparam = (size_t)nin * hidden + hidden + (size_t)hidden * hidden + hidden + hidden + 1;
    PALIAL_CK(net.params.ensure(sizeof(float) * net.nparam), "alloc");
    PALIAL_CK(net.grads.ensure(sizeof(float) * net.nparam), "alloc");
    PALIAL_CK(net.m.ensure(sizeof(float) * net.nparam), "alloc");
    PALIAL_CK(net.v.ensure(sizeof(float) * net.nparam), "alloc");
    // He initialisation (host RNG, seeded), zero biases
    std::vector<float> h(net.nparam, 0.f);
    std::mt19937_64 rng(seed);
    auto fill = [&](size_t off, int fan_in, size_t count) {
        std::normal_distribution<float> nd(0.f, std::sqrt(2.f / (float)fan_in));
        for (size_t i = 0; i < count; i++) h[off + i] = nd(rng);
    };
    fill(net.off_W1(), nin, (size_t)nin * hidden);
    fill(net.off_W2(), hidden, (size_t)hidden * hidden);
    fill(net.off_W3(), hidden, hidden);
    PALIAL_CK(cudaMemcpy(net.params.ptr, h.data(), sizeof(float) * net.nparam, cudaMemcpyHostToDevice), "init");
    PALIAL_CK(cudaMemset(net.m.ptr, 0, sizeof(float) * net.nparam), "init");
    PALIAL_CK(cudaMemset(net.v.ptr, 0, sizeof(float) * net.nparam), "init");
    net.step = 0;
    net.ready = true;
    return PALIAL_OK;
}

long long palial_mlp_param_count(void) { return net.ready ? (long long)net.nparam : 0; }

int palial_mlp_get_params(float *out) {
    palial_status *st = nullptr;
    if (!net.ready || !out) return PALIAL_ERR_ARG;
    PALIAL_CK(cudaMemcpy(out, net.params.ptr, sizeof(float) * net.nparam, cudaMemcpyDeviceToHost), "get");
    return PALIAL_OK;
}

int palial_mlp_set_params(const float *in) {
    palial_status *st = nullptr;
    if (!net.ready || !in) return PALIAL_ERR_ARG;
    PALIAL_CK(cudaMemcpy(net.params.ptr, in, sizeof(float) * net.nparam, cudaMemcpyHostToDevice), "set");
    return PALIAL_OK;
}

// Loss and gradient of the mean squared error on (X, y) (host arrays, n rows).
int palial_mlp_grad(const float *X, const float *y, int n, float *grads_out, float *loss_out) {
    palial_status *st = nullptr;
    if (!net.ready || !X || !y || n <= 0) return PALIAL_ERR_ARG;
    int rc = ensure_batch(n);
    if (rc) return rc;
    PALIAL_CK(cudaMemcpy(net.X.ptr, X, sizeof(float) * (size_t)n * net.nin, cudaMemcpyHostToDevice), "X");
    PALIAL_CK(cudaMemcpy(net.T.ptr, y, sizeof(float) * n, cudaMemcpyHostToDevice), "y");
    forward(n);
    backward(n);
    PALIAL_CK(cudaDeviceSynchronize(), "grad");
    if (grads_out) PALIAL_CK(cudaMemcpy(grads_out, net.grads.ptr, sizeof(float) * net.nparam, cudaMemcpyDeviceToHost), "g");
    if (loss_out) PALIAL_CK(cudaMemcpy(loss_out, net.loss.ptr, sizeof(float), cudaMemcpyDeviceToHost), "loss");
    return PALIAL_OK;
}

// Mini-batch Adam on (X, y): `epochs` passes in a seeded shuffled order; returns the mean loss
// of the last epoch.
int palial_mlp_train(const float *X, const float *y, int n, int epochs, int batch, float lr, uint64_t seed,
                     float *final_loss) {
    palial_status *st = nullptr;
    if (!net.ready || !X || !y || n <= 0 || batch <= 0) return PALIAL_ERR_ARG;
    int rc = ensure_batch(batch);
    if (rc) return rc;
    std::vector<int> order(n);
    for (int i = 0; i < n; i++) order[i] = i;
    std::mt19937_64 rng(seed);
    std::vector<float> xb((size_t)batch * net.nin), yb(batch);
    double epoch_loss = 0.0;
    for (int ep = 0; ep < epochs; ep++) {
        std::shuffle(order.begin(), order.end(), rng);
        epoch_loss = 0.0;
        int nb_ = 0;
        for (int s0 = 0; s0 + batch <= n; s0 += batch) {
            for (int i = 0; i < batch; i++) {
                const int r = order[s0 + i];
                memcpy(&xb[(size_t)i * net.nin], X + (size_t)r * net.nin, sizeof(float) * net.nin);
                yb[i] = y[r];
            }
            PALIAL_CK(cudaMemcpy(net.X.ptr, xb.data(), sizeof(float) * xb.size(), cudaMemcpyHostToDevice), "X");
            PALIAL_CK(cudaMemcpy(net.T.ptr, yb.data(), sizeof(float) * batch, cudaMemcpyHostToDevice), "y");
            forward(batch);
            backward(batch);
            net.step++;
            const float b1 = 0.9f, b2 = 0.999f;
            note_launch();
            mlpk::adam_kernel<<<64, 256>>>(net.params.as<float>(), net.grads.as<float>(), net.m.as<float>(),
                                           net.v.as<float>(), (int)net.nparam, lr, b1, b2, 1e-8f,
                                           1.f - std::pow(b1, (float)net.step), 1.f - std::pow(b2, (float)net.step));
            float l = 0;
            PALIAL_CK(cudaMemcpy(&l, net.loss.ptr, sizeof(float), cudaMemcpyDeviceToHost), "loss");
            epoch_loss += l;
            nb_++;
        }
        if (nb_) epoch_loss /= nb_;
    }
    PALIAL_CK(cudaGetLastError(), "train");
    if (final_loss) *final_loss = (float)epoch_loss;
    return PALIAL_OK;
}

int palial_mlp_predict(const float *X, int n, float *out) {
    palial_status *st = nullptr;
    if (!net.ready || !X || !out || n <= 0) return PALIAL_ERR_ARG;
    const int chunk = 65536;
    int rc = ensure_batch(std::min(n, chunk));
    if (rc) return rc;
    for (int s0 = 0; s0 < n; s0 += chunk) {
        const int b = std::min(chunk, n - s0);
        PALIAL_CK(cudaMemcpy(net.X.ptr, X + (size_t)s0 * net.nin, sizeof(float) * (size_t)b * net.nin,
                             cudaMemcpyHostToDevice), "X");
        forward(b);
        PALIAL_CK(cudaMemcpy(out + s0, net.Y.ptr, sizeof(float) * b, cudaMemcpyDeviceToHost), "Y");
    }
    return PALIAL_OK;
}

}  // extern "C"

// mpc_mlp.cu -- the learned step-size controller's network: a 16 -> 64 -> 64 -> 1 multilayer
// perceptron with SiLU activations, trained and evaluated by the kernels below.
//
// Weights (5313 floats, packed in this order): W1[64][16], b1[64], W2[64][64], b2[64], W3[64],
// b3.  Inputs are normalised per feature, x_n = (x - mean) / std, and the output is
// y = y_mean + y_std * out_n; the loss is the mean squared error of out_n against
// (y - y_mean) / y_std.  Training is minibatch Adam; every gradient is the exact
// derivative of that loss (tests compare it with an FP64 numpy statement of the same network).
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/mpc_gpu.h"

namespace {

constexpr int NI = MPC_NFEATURES, NH = 64;
constexpr int OFF_W1 = 0, OFF_B1 = NH * NI, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH, OFF_W3 = OFF_B2 + NH,
              OFF_B3 = OFF_W3 + NH, NW = OFF_B3 + 1;
static_assert(NW == 5313, "packed weight count");
constexpr int SB = 64;  // samples per gradient block

__device__ __forceinline__ float sigm(float z) { return 1.0f / (1.0f + expf(-z)); }
__device__ __forceinline__ float silu(float z) { return z * sigm(z); }
__device__ __forceinline__ float dsilu(float z) {
    const float s = sigm(z);
    return s * (1.0f + z * (1.0f - s));
}

// Loss and gradient over samples idx[b0 .. b0 + SB) of this block (all n when idx is null),
// accumulated into grad and loss with the 1/n of the mean.  norm = {mean[16], std[16], ym, ys}.
__global__ void __launch_bounds__(256) k_mlp_grad(const float* __restrict__ W, const float* __restrict__ X,
                                                  const float* __restrict__ Y, const int* __restrict__ idx, int n,
                                                  const float* __restrict__ norm, float* grad, float* loss) {
    extern __shared__ __align__(16) float sm[];
    float* w = sm;                 // NW
    float* x = w + NW + 3;         // SB x NI (16 B aligned: NW + 3 = 5316)
    float* z1 = x + SB * NI;       // SB x NH, later delta1
    float* h1 = z1 + SB * NH;      // SB x NH
    float* z2 = h1 + SB * NH;      // SB x NH, later delta2
    float* h2 = z2 + SB * NH;      // SB x NH
    float* d3 = h2 + SB * NH;      // SB
    const int tid = threadIdx.x, nt = blockDim.x;
    const int b0 = blockIdx.x * SB;
    const int nb = min(SB, n - b0);
    for (int k = tid; k < NW; k += nt) w[k] = W[k];
    for (int e = tid; e < SB * NI; e += nt) {
        const int b = e / NI, i = e % NI;
        float v = 0.0f;
        if (b < nb) {
            const int s = idx ? idx[b0 + b] : b0 + b;
            v = (X[(size_t)s * NI + i] - norm[i]) / norm[NI + i];
        }
        x[e] = v;
    }
    __syncthreads();
    for (int e = tid; e < SB * NH; e += nt) {
        const int b = e / NH, j = e % NH;
        float z = w[OFF_B1 + j];
        for (int i = 0; i < NI; i++) z = fmaf(w[OFF_W1 + j * NI + i], x[b * NI + i], z);
        z1[e] = z;
        h1[e] = silu(z);
    }
    __syncthreads();
    for (int e = tid; e < SB * NH; e += nt) {
        const int b = e / NH, k = e % NH;
        float z = w[OFF_B2 + k];
        for (int j = 0; j < NH; j++) z = fmaf(w[OFF_W2 + k * NH + j], h1[b * NH + j], z);
        z2[e] = z;
        h2[e] = silu(z);
    }
    __syncthreads();
    float lsum = 0.0f;
    if (tid < SB) {
        float d = 0.0f;
        if (tid < nb) {
            float o = w[OFF_B3];
            for (int k = 0; k < NH; k++) o = fmaf(w[OFF_W3 + k], h2[tid * NH + k], o);
            const int s = idx ? idx[b0 + tid] : b0 + tid;
            const float yn = (Y[s] - norm[2 * NI]) / norm[2 * NI + 1];
            const float r = o - yn;
            lsum = r * r / (float)n;
            d = 2.0f * r / (float)n;
        }
        d3[tid] = d;
    }
    __syncthreads();
    for (int e = tid; e < SB * NH; e += nt) {   // delta2 (into z2)
        const int b = e / NH, k = e % NH;
        z2[e] = d3[b] * w[OFF_W3 + k] * dsilu(z2[e]);
    }
    __syncthreads();
    for (int e = tid; e < SB * NH; e += nt) {   // delta1 (into z1)
        const int b = e / NH, j = e % NH;
        float a = 0.0f;
        for (int k = 0; k < NH; k++) a = fmaf(z2[b * NH + k], w[OFF_W2 + k * NH + j], a);
        z1[e] = a * dsilu(z1[e]);
    }
    __syncthreads();
    // weight gradients: sums over the block's samples (padded samples carry zero deltas)
    for (int e = tid; e < NW; e += nt) {
        float g = 0.0f;
        if (e < OFF_B1) {
            const int j = e / NI, i = e % NI;
            for (int b = 0; b < SB; b++) g = fmaf(z1[b * NH + j], x[b * NI + i], g);
        } else if (e < OFF_W2) {
            const int j = e - OFF_B1;
            for (int b = 0; b < SB; b++) g += z1[b * NH + j];
        } else if (e < OFF_B2) {
            const int k = (e - OFF_W2) / NH, j = (e - OFF_W2) % NH;
            for (int b = 0; b < SB; b++) g = fmaf(z2[b * NH + k], h1[b * NH + j], g);
        } else if (e < OFF_W3) {
            const int k = e - OFF_B2;
            for (int b = 0; b < SB; b++) g += z2[b * NH + k];
        } else if (e < OFF_B3) {
            const int k = e - OFF_W3;
            for (int b = 0; b < SB; b++) g = fmaf(d3[b], h2[b * NH + k], g);
        } else {
            for (int b = 0; b < SB; b++) g += d3[b];
        }
        atomicAdd(&grad[e], g);
    }
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if ((tid & 31) == 0 && tid < SB) atomicAdd(loss, lsum);
}

// Adam (Kingma and Ba, 2015) with bias correction; c1 = 1 - beta1^t, c2 = 1 - beta2^t
__global__ void k_adam(float* W, const float* __restrict__ g, float* m, float* v, int n, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float gk = g[k];
    const float mk = b1 * m[k] + (1.0f - b1) * gk;
    const float vk = b2 * v[k] + (1.0f - b2) * gk * gk;
    m[k] = mk;
    v[k] = vk;
    W[k] -= lr * (mk / c1) / (sqrtf(vk / c2) + eps);
}

// Inference, one sample per thread: y = ym + ys * net((x - mean) / std)
__global__ void __launch_bounds__(128) k_mlp_predict(const float* __restrict__ W, const float* __restrict__ X, int n,
                                                     const float* __restrict__ norm, float* __restrict__ Y) {
    __shared__ float w[NW];
    for (int k = threadIdx.x; k < NW; k += blockDim.x) w[k] = W[k];
    __syncthreads();
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= n) return;
    float x[NI];
#pragma unroll
    for (int i = 0; i < NI; i++) x[i] = (X[(size_t)s * NI + i] - norm[i]) / norm[NI + i];
    float h1[NH];
#pragma unroll 4
    for (int j = 0; j < NH; j++) {
        float z = w[OFF_B1 + j];
#pragma unroll
        for (int i = 0; i < NI; i++) z = fmaf(w[OFF_W1 + j * NI + i], x[i], z);
        h1[j] = silu(z);
    }
    float o = w[OFF_B3];
    for (int k = 0; k < NH; k++) {
        float z = w[OFF_B2 + k];
#pragma unroll
        for (int j = 0; j < NH; j++) z = fmaf(w[OFF_W2 + k * NH + j], h1[j], z);
        o = fmaf(w[OFF_W3 + k], silu(z), o);
    }
    Y[s] = norm[2 * NI] + norm[2 * NI + 1] * o;
}

constexpr size_t kGradSmem = sizeof(float) * (NW + 3 + SB * NI + 4 * SB * NH + SB);

uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
double unit(uint64_t& s) { return ((splitmix(s) >> 11) + 0.5) / 9007199254740992.0; }

thread_local std::string g_mlp_err;
int mlp_fail(int code, const char* what, cudaError_t e = cudaSuccess) {
    char buf[256];
    if (e != cudaSuccess) snprintf(buf, sizeof buf, "mlp: %s: %s", what, cudaGetErrorString(e));
    else snprintf(buf, sizeof buf, "mlp: %s", what);
    g_mlp_err = buf;
    fprintf(stderr, "%s\n", buf);
    return code;
}
#define MCK(call, what)                                              \
    do {                                                             \
        cudaError_t _e = (call);                                     \
        if (_e != cudaSuccess) return mlp_fail(MPC_ERR_CUDA, what, _e); \
    } while (0)

}  // namespace

struct mpc_mlp {
    float* W = nullptr;     // device weights
    float* m = nullptr;     // Adam moments
    float* v = nullptr;
    float* g = nullptr;     // gradient
    float* loss = nullptr;  // device loss accumulator
    float* norm = nullptr;  // device {mean[16], std[16], y_mean, y_std}
    float hnorm[2 * NI + 2];
    float* dio = nullptr;   // device buffer of one sample and its prediction (predict1)
    float* hio = nullptr;   // pinned host copy of it
    long t = 0;             // Adam steps taken
    cudaStream_t st = nullptr;
    bool smem_ready = false;
};

extern "C" {

int mpc_mlp_num_weights(void) { return NW; }

int mpc_mlp_destroy(mpc_mlp* m) {
    if (!m) return MPC_OK;
    if (m->st) cudaStreamSynchronize(m->st);
    for (float* p : {m->W, m->m, m->v, m->g, m->loss, m->norm, m->dio})
        if (p) cudaFree(p);
    if (m->hio) cudaFreeHost(m->hio);
    if (m->st) cudaStreamDestroy(m->st);
    delete m;
    return MPC_OK;
}

int mpc_mlp_create(mpc_mlp** out, unsigned long long seed) {
    if (!out) return mlp_fail(MPC_ERR_ARG, "null argument");
    *out = nullptr;
    mpc_mlp* m = new mpc_mlp();
    cudaError_t e = cudaStreamCreateWithFlags(&m->st, cudaStreamNonBlocking);
    for (float** p : {&m->W, &m->m, &m->v, &m->g})
        if (e == cudaSuccess) e = cudaMalloc(p, sizeof(float) * NW);
    if (e == cudaSuccess) e = cudaMalloc(&m->loss, sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&m->norm, sizeof m->hnorm);
    if (e == cudaSuccess) e = cudaMalloc(&m->dio, sizeof(float) * (NI + 1));
    if (e == cudaSuccess) e = cudaMallocHost(&m->hio, sizeof(float) * (NI + 1));
    if (e != cudaSuccess) {
        mpc_mlp_destroy(m);
        cudaGetLastError();
        return mlp_fail(MPC_ERR_NOMEM, "device buffers", e);
    }
    // uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)) weights and biases, from splitmix64(seed)
    std::vector<float> w(NW);
    uint64_t s = seed;
    for (int k = 0; k < NW; k++) {
        const double fan = k < OFF_W2 ? NI : (k < OFF_W3 ? NH : NH);
        w[k] = (float)((2.0 * unit(s) - 1.0) / sqrt(fan));
    }
    for (int i = 0; i < 2 * NI + 2; i++) m->hnorm[i] = (i < NI || i == 2 * NI) ? 0.0f : 1.0f;
    e = cudaMemcpy(m->W, w.data(), sizeof(float) * NW, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(m->norm, m->hnorm, sizeof m->hnorm, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(m->m, 0, sizeof(float) * NW);
    if (e == cudaSuccess) e = cudaMemset(m->v, 0, sizeof(float) * NW);
    if (e != cudaSuccess) {
        mpc_mlp_destroy(m);
        return mlp_fail(MPC_ERR_CUDA, "initialisation", e);
    }
    *out = m;
    return MPC_OK;
}

int mpc_mlp_set_normalization(mpc_mlp* m, const float* mean, const float* stdv, float y_mean, float y_std) {
    if (!m || !mean || !stdv) return mlp_fail(MPC_ERR_ARG, "null argument");
    for (int i = 0; i < NI; i++) {
        if (!(stdv[i] > 0)) return mlp_fail(MPC_ERR_ARG, "feature scales must be positive");
        m->hnorm[i] = mean[i];
        m->hnorm[NI + i] = stdv[i];
    }
    if (!(y_std > 0)) return mlp_fail(MPC_ERR_ARG, "target scale must be positive");
    m->hnorm[2 * NI] = y_mean;
    m->hnorm[2 * NI + 1] = y_std;
    MCK(cudaMemcpy(m->norm, m->hnorm, sizeof m->hnorm, cudaMemcpyHostToDevice), "normalisation");
    return MPC_OK;
}

int mpc_mlp_get_normalization(mpc_mlp* m, float* out) {
    if (!m || !out) return mlp_fail(MPC_ERR_ARG, "null argument");
    memcpy(out, m->hnorm, sizeof m->hnorm);
    return MPC_OK;
}

int mpc_mlp_get_weights(mpc_mlp* m, float* w) {
    if (!m || !w) return mlp_fail(MPC_ERR_ARG, "null argument");
    MCK(cudaStreamSynchronize(m->st), "sync");
    MCK(cudaMemcpy(w, m->W, sizeof(float) * NW, cudaMemcpyDeviceToHost), "D2H weights");
    return MPC_OK;
}

int mpc_mlp_set_weights(mpc_mlp* m, const float* w) {
    if (!m || !w) return mlp_fail(MPC_ERR_ARG, "null argument");
    MCK(cudaStreamSynchronize(m->st), "sync");
    MCK(cudaMemcpy(m->W, w, sizeof(float) * NW, cudaMemcpyHostToDevice), "H2D weights");
    MCK(cudaMemset(m->m, 0, sizeof(float) * NW), "reset Adam");
    MCK(cudaMemset(m->v, 0, sizeof(float) * NW), "reset Adam");
    m->t = 0;
    return MPC_OK;
}

static int grad_launch(mpc_mlp* m, const float* dX, const float* dY, const int* didx, int n) {
    if (!m->smem_ready) {
        MCK(cudaFuncSetAttribute(k_mlp_grad, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGradSmem), "smem attr");
        m->smem_ready = true;
    }
    MCK(cudaMemsetAsync(m->g, 0, sizeof(float) * NW, m->st), "memset grad");
    MCK(cudaMemsetAsync(m->loss, 0, sizeof(float), m->st), "memset loss");
    k_mlp_grad<<<(n + SB - 1) / SB, 256, kGradSmem, m->st>>>(m->W, dX, dY, didx, n, m->norm, m->g, m->loss);
    MCK(cudaGetLastError(), "k_mlp_grad");
    return MPC_OK;
}

int mpc_mlp_loss_grad(mpc_mlp* m, const float* X, const float* y, int n, float* grad, float* loss) {
    if (!m || !X || !y || n <= 0 || !grad || !loss) return mlp_fail(MPC_ERR_ARG, "null argument or empty set");
    float *dX = nullptr, *dY = nullptr;
    MCK(cudaMalloc(&dX, sizeof(float) * (size_t)n * NI), "cudaMalloc X");
    cudaError_t e = cudaMalloc(&dY, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dX, X, sizeof(float) * (size_t)n * NI, cudaMemcpyHostToDevice, m->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dY, y, sizeof(float) * n, cudaMemcpyHostToDevice, m->st);
    int rc = (e == cudaSuccess) ? grad_launch(m, dX, dY, nullptr, n) : mlp_fail(MPC_ERR_CUDA, "H2D data", e);
    if (rc == MPC_OK) {
        e = cudaMemcpyAsync(grad, m->g, sizeof(float) * NW, cudaMemcpyDeviceToHost, m->st);
        if (e == cudaSuccess) e = cudaMemcpyAsync(loss, m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(m->st);
        if (e != cudaSuccess) rc = mlp_fail(MPC_ERR_CUDA, "gradient", e);
    }
    cudaStreamSynchronize(m->st);
    cudaFree(dX);
    if (dY) cudaFree(dY);
    return rc;
}

int mpc_mlp_train(mpc_mlp* m, const float* X, const float* y, int n, int epochs, int batch, float lr,
                  unsigned long long seed, float* final_loss) {
    if (!m || !X || !y || n <= 0 || epochs <= 0 || batch <= 0 || !(lr > 0)) return mlp_fail(MPC_ERR_ARG, "bad argument");
    float *dX = nullptr, *dY = nullptr;
    int* didx = nullptr;
    MCK(cudaMalloc(&dX, sizeof(float) * (size_t)n * NI), "cudaMalloc X");
    cudaError_t e = cudaMalloc(&dY, sizeof(float) * n);
    if (e == cudaSuccess) e = cudaMalloc(&didx, sizeof(int) * n);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dX, X, sizeof(float) * (size_t)n * NI, cudaMemcpyHostToDevice, m->st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dY, y, sizeof(float) * n, cudaMemcpyHostToDevice, m->st);
    int rc = (e == cudaSuccess) ? MPC_OK : mlp_fail(MPC_ERR_CUDA, "training data", e);
    std::vector<int> perm(n);
    for (int i = 0; i < n; i++) perm[i] = i;
    uint64_t s = seed;
    std::vector<float> epoch_loss;
    std::vector<float> bl;
    for (int ep = 0; ep < epochs && rc == MPC_OK; ep++) {
        for (int i = n - 1; i > 0; i--) std::swap(perm[i], perm[splitmix(s) % (uint64_t)(i + 1)]);   // Fisher-Yates
        e = cudaMemcpyAsync(didx, perm.data(), sizeof(int) * n, cudaMemcpyHostToDevice, m->st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(m->st);   // perm is rewritten next epoch
        if (e != cudaSuccess) {
            rc = mlp_fail(MPC_ERR_CUDA, "permutation", e);
            break;
        }
        const int nbat = (n + batch - 1) / batch;
        bl.assign(nbat, 0.0f);
        for (int b = 0; b < nbat && rc == MPC_OK; b++) {
            const int b0 = b * batch, nb = std::min(batch, n - b0);
            rc = grad_launch(m, dX, dY, didx + b0, nb);
            if (rc) break;
            m->t++;
            const float c1 = 1.0f - powf(0.9f, (float)m->t), c2 = 1.0f - powf(0.999f, (float)m->t);
            k_adam<<<(NW + 255) / 256, 256, 0, m->st>>>(m->W, m->g, m->m, m->v, NW, lr, 0.9f, 0.999f, 1e-8f, c1, c2);
            e = cudaGetLastError();
            if (e == cudaSuccess) e = cudaMemcpyAsync(&bl[b], m->loss, sizeof(float), cudaMemcpyDeviceToHost, m->st);
            if (e != cudaSuccess) rc = mlp_fail(MPC_ERR_CUDA, "Adam step", e);
        }
        if (rc == MPC_OK && (e = cudaStreamSynchronize(m->st)) != cudaSuccess) rc = mlp_fail(MPC_ERR_CUDA, "epoch", e);
        double tot = 0.0;
        for (int b = 0; b < nbat; b++) tot += (double)bl[b] * std::min(batch, n - b * batch);
        epoch_loss.push_back((float)(tot / n));
    }
    cudaStreamSynchronize(m->st);
    cudaFree(dX);
    if (dY) cudaFree(dY);
    if (didx) cudaFree(didx);
    if (rc == MPC_OK && final_loss) *final_loss = epoch_loss.empty() ? 0.0f : epoch_loss.back();
    return rc;
}

int mpc_mlp_predict(mpc_mlp* m, const float* X, int n, float* y) {
    if (!m || !X || n <= 0 || !y) return mlp_fail(MPC_ERR_ARG, "null argument or empty set");
    float *dX = nullptr, *dY = nullptr;
    MCK(cudaMalloc(&dX, sizeof(float) * ((size_t)n * NI + n)), "cudaMalloc");
    dY = dX + (size_t)n * NI;
    cudaError_t e = cudaMemcpyAsync(dX, X, sizeof(float) * (size_t)n * NI, cudaMemcpyHostToDevice, m->st);
    if (e == cudaSuccess) {
        k_mlp_predict<<<(n + 127) / 128, 128, 0, m->st>>>(m->W, dX, n, m->norm, dY);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(y, dY, sizeof(float) * n, cudaMemcpyDeviceToHost, m->st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(m->st);
    cudaStreamSynchronize(m->st);
    cudaFree(dX);
    if (e != cudaSuccess) return mlp_fail(MPC_ERR_CUDA, "predict", e);
    return MPC_OK;
}

int mpc_mlp_predict1(mpc_mlp* m, const float* x, float* y) {
    if (!m || !x || !y) return mlp_fail(MPC_ERR_ARG, "null argument");
    memcpy(m->hio, x, sizeof(float) * NI);
    MCK(cudaMemcpyAsync(m->dio, m->hio, sizeof(float) * NI, cudaMemcpyHostToDevice, m->st), "H2D sample");
    k_mlp_predict<<<1, 128, 0, m->st>>>(m->W, m->dio, 1, m->norm, m->dio + NI);
    MCK(cudaGetLastError(), "k_mlp_predict");
    MCK(cudaMemcpyAsync(m->hio + NI, m->dio + NI, sizeof(float), cudaMemcpyDeviceToHost, m->st), "D2H prediction");
    MCK(cudaStreamSynchronize(m->st), "predict1");
    *y = m->hio[NI];
    return MPC_OK;
}

}  // extern "C"

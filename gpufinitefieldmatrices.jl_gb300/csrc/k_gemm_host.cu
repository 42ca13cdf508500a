// k_gemm_host.cu -- C = A*B mod N with A, B and C in host memory, the copies
// overlapped with the products.
//
// A is cut into row blocks and B into column blocks (about 2048 wide).  The
// blocks go to the device on one copy stream, A_0, B_0, A_1, B_1, ...; each
// product block C_ij = A_i B_j mod N (digit splits of A_i and B_j on first use,
// then the limb tensor-core GEMM) runs on one of two compute streams as soon as
// its two blocks are resident, in the order of max(i, j), so the products
// start after the first block pair and the copies of the later blocks hide
// behind them; the second compute stream lets a product's first tiles fill the
// SMs its predecessor's last wave leaves idle.  Each finished C_ij goes back on
// a second copy stream.  Only the first block pair's copy and the last block's
// copy back stay exposed.  The host buffers should be page-locked for the
// copies to run asynchronously.
#include "gffm_common.cuh"
#include "kara_host.h"
#include "limb_host.h"

#include <algorithm>
#include <map>
#include <mutex>
#include <vector>

namespace {

using gffm::set_error;

struct HostStreams {
    cudaStream_t in = nullptr, out = nullptr, c[2] = {nullptr, nullptr};
};

// per-device streams, created on first use and kept for the life of the process
std::mutex g_mu;
std::map<int, HostStreams> g_streams;

int streams_for(HostStreams *hs) {
    int dev = 0;
    GFFM_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(g_mu);
    auto it = g_streams.find(dev);
    if (it == g_streams.end()) {
        HostStreams s;
        GFFM_CUDA(cudaStreamCreateWithFlags(&s.in, cudaStreamNonBlocking));
        GFFM_CUDA(cudaStreamCreateWithFlags(&s.out, cudaStreamNonBlocking));
        GFFM_CUDA(cudaStreamCreateWithFlags(&s.c[0], cudaStreamNonBlocking));
        GFFM_CUDA(cudaStreamCreateWithFlags(&s.c[1], cudaStreamNonBlocking));
        it = g_streams.emplace(dev, s).first;
    }
    *hs = it->second;
    return GFFM_OK;
}

constexpr int64_t kAlign = 1024;

// Block boundaries: rows of A in multiples of 128, columns of B in multiples of 64,
// about 2048 wide (a 2048 x 2048 product block is 512 output tiles, over three waves
// of SMs).  Narrower first blocks would start the products sooner but run them
// below full waves, which costs more than it saves (1024-wide first blocks: 12.06
// instead of 11.58 ms at 8192^3).
std::vector<int64_t> cuts(int64_t len, int64_t quantum) {
    std::vector<int64_t> c{0};
    const int64_t t = std::max<int64_t>(1, (len + 2047) / 2048);
    const int64_t w = gffm::round_up((len + t - 1) / t, quantum);
    for (int64_t at = 0; at < len;) c.push_back(at = std::min(len, at + w));
    return c;
}

struct Blocks {
    std::vector<int64_t> ra, cb;   // row cuts of A, column cuts of B (first 0, last m / n)
    int na, nb;
};
Blocks blocks_for(int64_t m, int64_t n, int64_t col_quantum) {
    Blocks b;
    b.ra = cuts(m, 128);
    b.cb = cuts(n, col_quantum);
    b.na = (int)b.ra.size() - 1;
    b.nb = (int)b.cb.size() - 1;
    return b;
}

// device workspace: staging copies of A, B, C (Float64, leading dimensions rounded
// to 32) and the digit planes of every block of A and of B
struct HostLayout {
    Blocks b;
    int bits, tile_n, form;
    int64_t lda_d, ldb_d, ldc_d;
    size_t off_a, off_b, off_c;
    std::vector<size_t> off_da, off_db;
    size_t total;
};

HostLayout host_layout(int64_t m, int64_t n, int64_t k, int64_t N) {
    HostLayout h;
    int ctas = 0;
    limb::tuned_for(m, n, k, N, &h.bits, &ctas, &h.tile_n, &h.form);
    if (h.form == limb::FORM_KARATSUBA && !kara::applies(N)) h.form = limb::FORM_SCHOOLBOOK;
    h.form = limb::resolve_form(h.form, h.bits, h.tile_n, N, k);
    const bool kf = h.form == limb::FORM_KARATSUBA;
    h.b = blocks_for(m, n, kf ? 128 : 64);
    h.lda_d = gffm::round_up(std::max<int64_t>(m, 1), 32);
    h.ldb_d = gffm::round_up(std::max<int64_t>(k, 1), 32);
    h.ldc_d = h.lda_d;
    size_t off = 0;
    auto take = [&](size_t bytes) {
        const size_t o = off;
        off = (size_t)gffm::round_up((int64_t)(off + bytes), kAlign);
        return o;
    };
    h.off_a = take((size_t)h.lda_d * (size_t)std::max<int64_t>(k, 1) * 8);
    h.off_b = take((size_t)h.ldb_d * (size_t)std::max<int64_t>(n, 1) * 8);
    h.off_c = take((size_t)h.ldc_d * (size_t)std::max<int64_t>(n, 1) * 8);
    if (k > 0) {
        for (int i = 0; i < h.b.na; i++) {
            const int64_t rows = h.b.ra[i + 1] - h.b.ra[i];
            h.off_da.push_back(take(kf ? kara::layout(rows, 1, k).a_bytes
                                       : limb::layout_bits(rows, 1, k, N, h.bits).a_bytes));
        }
        for (int j = 0; j < h.b.nb; j++) {
            const int64_t cols = h.b.cb[j + 1] - h.b.cb[j];
            h.off_db.push_back(take(kf ? kara::layout(1, cols, k).b_bytes
                                       : limb::layout_bits(1, cols, k, N, h.bits).b_bytes));
        }
    }
    h.total = off;
    return h;
}

// events of one call, destroyed when the call returns (the pending ones are
// released by the runtime once they complete)
struct Events {
    std::vector<cudaEvent_t> ev;
    ~Events() {
        for (cudaEvent_t e : ev) cudaEventDestroy(e);
    }
    int make(cudaEvent_t *e) {
        GFFM_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
        ev.push_back(*e);
        return GFFM_OK;
    }
};

// the copies, splits and products of one call on the internal streams (which wait for e0)
int enqueue(const HostLayout &h, const HostStreams &hs, uint8_t *base, int64_t m, int64_t n, int64_t k,
            const double *hA, int64_t lda, const double *hB, int64_t ldb, double *hC, int64_t ldc, int64_t N,
            Events &evs) {
    int st = GFFM_OK;
    double *dA = reinterpret_cast<double *>(base + h.off_a);
    double *dB = reinterpret_cast<double *>(base + h.off_b);
    double *dC = reinterpret_cast<double *>(base + h.off_c);
    if (k == 0) {   // C = 0
        GFFM_CUDA(cudaMemset2DAsync(dC, (size_t)h.ldc_d * 8, 0, (size_t)m * 8, (size_t)n, hs.out));
        GFFM_CUDA(cudaMemcpy2DAsync(hC, (size_t)ldc * 8, dC, (size_t)h.ldc_d * 8, (size_t)m * 8, (size_t)n,
                                    cudaMemcpyDeviceToHost, hs.out));
        return GFFM_OK;
    }

    const Blocks &b = h.b;
    auto rows_of = [&](int i) { return b.ra[i + 1] - b.ra[i]; };
    auto cols_of = [&](int j) { return b.cb[j + 1] - b.cb[j]; };
    std::vector<cudaEvent_t> a_in(b.na), b_in(b.nb), a_sp(b.na), b_sp(b.nb);
    for (auto *v : {&a_in, &a_sp})
        for (auto &e : *v)
            if ((st = evs.make(&e))) return st;
    for (auto *v : {&b_in, &b_sp})
        for (auto &e : *v)
            if ((st = evs.make(&e))) return st;

    // copies in: A_0, B_0, A_1, B_1, ...
    for (int q = 0; q < std::max(b.na, b.nb); q++) {
        if (q < b.na) {
            const int64_t r0 = b.ra[q];
            GFFM_CUDA(cudaMemcpy2DAsync(dA + r0, (size_t)h.lda_d * 8, hA + r0, (size_t)lda * 8, (size_t)rows_of(q) * 8,
                                        (size_t)k, cudaMemcpyHostToDevice, hs.in));
            GFFM_CUDA(cudaEventRecord(a_in[q], hs.in));
        }
        if (q < b.nb) {
            const int64_t c0 = b.cb[q];
            GFFM_CUDA(cudaMemcpy2DAsync(dB + c0 * h.ldb_d, (size_t)h.ldb_d * 8, hB + c0 * ldb, (size_t)ldb * 8,
                                        (size_t)k * 8, (size_t)cols_of(q), cudaMemcpyHostToDevice, hs.in));
            GFFM_CUDA(cudaEventRecord(b_in[q], hs.in));
        }
    }

    // products in the order of max(i, j); splits on the stream of their first use
    std::vector<std::pair<int, int>> order;
    for (int q = 0; q < std::max(b.na, b.nb); q++) {
        if (q < b.na)   // A_q arrives before B_q
            for (int j = 0; j < b.nb && j < q; j++) order.emplace_back(q, j);
        if (q < b.nb)
            for (int i = 0; i < b.na && i <= q; i++) order.emplace_back(i, q);
    }
    std::vector<int> a_on(b.na, -1), b_on(b.nb, -1);
    int which = 0;
    for (const auto &ij : order) {
        const int i = ij.first, j = ij.second;
        const int64_t rows = rows_of(i), cols = cols_of(j);
        cudaStream_t c = hs.c[which];
        const bool kf = h.form == limb::FORM_KARATSUBA;
        limb::Layout g = limb::layout_bits(rows, cols, k, N, h.bits);
        g.bn = h.tile_n;
        const kara::Layout kg = kara::layout(rows, cols, k);
        __half *Ad = reinterpret_cast<__half *>(base + h.off_da[i]);
        __half *Bd = reinterpret_cast<__half *>(base + h.off_db[j]);
        if (a_on[i] < 0) {
            GFFM_CUDA(cudaStreamWaitEvent(c, a_in[i], 0));
            st = kf ? kara::split_a<double>(dA + b.ra[i], h.lda_d, rows, k, Ad, kg, N, c)
                    : limb::split_a<double>(dA + b.ra[i], h.lda_d, rows, k, Ad, g, N, c);
            if (st) return st;
            GFFM_CUDA(cudaEventRecord(a_sp[i], c));
            a_on[i] = which;
        } else if (a_on[i] != which) {
            GFFM_CUDA(cudaStreamWaitEvent(c, a_sp[i], 0));
        }
        if (b_on[j] < 0) {
            GFFM_CUDA(cudaStreamWaitEvent(c, b_in[j], 0));
            st = kf ? kara::split_b<double>(dB + b.cb[j] * h.ldb_d, h.ldb_d, k, cols, Bd, kg, N, c)
                    : limb::split_b<double>(dB + b.cb[j] * h.ldb_d, h.ldb_d, k, cols, Bd, g, N, c);
            if (st) return st;
            GFFM_CUDA(cudaEventRecord(b_sp[j], c));
            b_on[j] = which;
        } else if (b_on[j] != which) {
            GFFM_CUDA(cudaStreamWaitEvent(c, b_sp[j], 0));
        }
        double *Cij = dC + b.ra[i] + b.cb[j] * h.ldc_d;
        st = kf ? kara::gemm_digits(kg, Ad, Bd, rows, cols, k, N, Cij, h.ldc_d, limb::EPI_STORE_F64, 0, c)
                : limb::gemm_digits(g, Ad, Bd, rows, cols, k, N, Cij, h.ldc_d, limb::EPI_STORE_F64, 0, c);
        if (st) return st;
        cudaEvent_t e_c;
        if ((st = evs.make(&e_c))) return st;
        GFFM_CUDA(cudaEventRecord(e_c, c));
        GFFM_CUDA(cudaStreamWaitEvent(hs.out, e_c, 0));
        GFFM_CUDA(cudaMemcpy2DAsync(hC + b.ra[i] + b.cb[j] * ldc, (size_t)ldc * 8, Cij, (size_t)h.ldc_d * 8,
                                    (size_t)rows * 8, (size_t)cols, cudaMemcpyDeviceToHost, hs.out));
        which ^= 1;
    }
    return GFFM_OK;
}

int matmul_host(int64_t m, int64_t n, int64_t k, const double *hA, int64_t lda, const double *hB, int64_t ldb,
                double *hC, int64_t ldc, int64_t N, void *ws, size_t ws_bytes, gffm_stream_t stream) {
    int st = limb::check_args(m, n, k, lda, ldb, ldc, N);
    if (st) return st;
    if (m == 0 || n == 0) return GFFM_OK;
    if (!hC || (k > 0 && (!hA || !hB))) return set_error(GFFM_ERR_ARG, "null data pointer");
    st = gffm::check_device();
    if (st) return st;
    cudaStream_t s0 = gffm::as_stream(stream);
    HostStreams hs;
    st = streams_for(&hs);
    if (st) return st;
    const HostLayout h = host_layout(m, n, k, N);
    gffm::Scratch scr;
    st = scr.acquire(ws, ws_bytes, h.total, s0);
    if (st) return st;
    Events evs;
    cudaEvent_t e0;
    if ((st = evs.make(&e0))) return st;
    GFFM_CUDA(cudaEventRecord(e0, s0));
    const cudaStream_t inner[4] = {hs.in, hs.out, hs.c[0], hs.c[1]};
    for (cudaStream_t s : inner) GFFM_CUDA(cudaStreamWaitEvent(s, e0, 0));
    st = enqueue(h, hs, static_cast<uint8_t *>(scr.ptr), m, n, k, hA, lda, hB, ldb, hC, ldc, N, evs);
    // the caller's stream (and the workspace's release on it) follows all of it, even
    // after an error part way through
    for (cudaStream_t s : inner) {
        cudaEvent_t e;
        int st2 = evs.make(&e);
        if (!st2 && cudaEventRecord(e, s) == cudaSuccess) cudaStreamWaitEvent(s0, e, 0);
        else if (!st) st = st2 ? st2 : set_error(GFFM_ERR_CUDA, "cannot join the copy and product streams");
    }
    return st;
}

}  // namespace

extern "C" {

int gffm_matmul_host_workspace_size(int64_t m, int64_t n, int64_t k, int64_t N, size_t *bytes) {
    if (!bytes) return set_error(GFFM_ERR_ARG, "bytes is NULL");
    int st = limb::check_args(m, n, k, m > 1 ? m : 1, k > 1 ? k : 1, m > 1 ? m : 1, N);
    if (st) return st;
    *bytes = (m == 0 || n == 0) ? 0 : host_layout(m, n, k, N).total;
    return GFFM_OK;
}

int gffm_matmul_host_f64(int64_t m, int64_t n, int64_t k, const double *A, int64_t lda, const double *B, int64_t ldb,
                         double *C, int64_t ldc, int64_t N, void *ws, size_t ws_bytes, gffm_stream_t stream) {
    return matmul_host(m, n, k, A, lda, B, ldb, C, ldc, N, ws, ws_bytes, stream);
}

}  // extern "C"

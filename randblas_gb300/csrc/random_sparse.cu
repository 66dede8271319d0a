// random_sparse.cu -- random_coo / random_csr / random_csc (RandBLAS/sparse_data/random_matrix.hh:
// 135-355) on the GPU, with the reference's nonzero positions, order, values and next state.
//
// The reference draws from one sequential word stream (PhiloxStream, random_matrix.hh:63-121):
// word w is lane w mod 4 of Philox at counter seed + w / 4.  A geometric draw takes one word
// (floor(log(1 - u) / log(1 - p)), u = w * 2^-32 + 2^-33 in double); a Gaussian takes a fresh
// word pair (boxmuller, first value) or returns the second value of the previous pair.  Nonzero
// k's value is therefore always a value of the pair drawn right after the skip that created
// nonzero k - (k mod 2); what varies is only where the words sit.
//
// COO: one geometric process over the row-major linear index.  Per two nonzeros the stream
// holds the value pair and then the two skip words, so nonzero k's skip and pair have fixed
// positions, its linear index is a prefix sum of skips (a saturating scan), and nonzero k
// exists iff that index is below m * n.
//
// CSR / CSC: every row (column) opens with its own geometric draw, so where row i's words start
// depends on the nonzero counts of all rows before it.  A row start is a node
// (word position p, parity pi of the number of nonzeros before it).  From a node the row's skip
// words visit a fixed residue pair mod 4 -- steps 3, 1, 3, 1 when pi = 0 (the first nonzero
// draws a pair), 1, 3, 1, 3 when pi = 1 -- so the row ends at the first crossing of a prefix
// sum of (1 + skip) over that residue class, found by a galloping search.  That gives every
// node its successor (the next row's start).  The true row starts are the chain from node
// (0, even), marked by pointer jumping in ceil(log2(rows)) rounds; a scan of the row counts
// gives the pointers, and each nonzero's column and value pair follow from its row's start.
//
// CUDA's double log can differ from the host library's in the last place, which changes a
// skip only when the quotient lies within a few ulp of an integer (about 1e-14 per draw).
// Every skip the matrix uses is checked, and the number of such near-ties is reported
// (rbg_random_sparse_info); results are bit-identical to the reference whenever it is zero.
#include <cub/device/device_scan.cuh>

#include <algorithm>
#include <cmath>
#include <string>

#include "rbg_internal.h"

namespace rbg {
namespace {

constexpr int kThreads = 256;

// CTAs of kThreads for a grid-stride loop over n items
inline int ctas(int64_t n) { return grid_stride_ctas(n, kThreads); }
constexpr uint32_t kNearTie = 0x80000000u;  // flag bit of a stored compressed-path skip
constexpr uint32_t kSkipMask = 0x7fffffffu;
// relative distance to an integer below which host and device logarithms may floor
// differently (each log is within one ulp; the quotient is rounded once)
constexpr double kNearIntRel = 0x1p-48;
// largest word budget of the compressed path: node ids 2 * words + parity fit in int32
constexpr int64_t kMaxWords = (int64_t(1) << 30) - 64;

struct Status {
    int64_t consumed;   // stream words the reference's loop draws
    int64_t ambiguous;  // skips within kNearIntRel of an integer
    int64_t nnz;        // COO: number of nonzeros (-1: candidates exhausted)
    int32_t overflow;   // the chain ran past the word budget
    int32_t broken;     // a row's end is not in its start's residue class (an internal error)
};

__device__ __forceinline__ uint32_t lane_of(const uint4 &r, int l) {
    return l == 0 ? r.x : l == 1 ? r.y : l == 2 ? r.z : r.w;
}

__device__ __forceinline__ uint32_t stream_word(const DevState &s, int64_t w) {
    return lane_of(philox(ctr_add(s.ctr, (uint64_t)w >> 2), s.key), (int)(w & 3));
}

// boxmuller on stream words (a, a + 1) -- the pair may straddle two Philox blocks
__device__ __forceinline__ void gaussian_pair(const DevState &s, int64_t a, float &first,
                                              float &second) {
    const uint4 r = philox(ctr_add(s.ctr, (uint64_t)a >> 2), s.key);
    const int l = (int)(a & 3);
    const uint32_t u0 = lane_of(r, l);
    const uint32_t u1 = l < 3 ? lane_of(r, l + 1)
                              : philox(ctr_add(s.ctr, ((uint64_t)a >> 2) + 1), s.key).x;
    boxmuller(u0, u1, first, second);
}

// PhiloxStream::geometric (random_matrix.hh:109-113); near_tie as described above.
__device__ __forceinline__ int64_t geometric(uint32_t w, double log_1_minus_p, bool &near_tie) {
    const double u = __dadd_rn(__dmul_rn((double)w, 0x1p-32), 0x1p-33);  // exact
    const double y = __ddiv_rn(log(__dsub_rn(1.0, u)), log_1_minus_p);
    const double f = floor(y);
    near_tie = (y - f) <= kNearIntRel * y || (f + 1.0 - y) <= kNearIntRel * y;
    return (int64_t)f;
}

// ----------------------------------------------------------------- compressed (CSR / CSC)
// Residue class b (0..3) holds the word positions o + 4h and o + 4h + 1, o = b - 1; rank r of
// the class is position 4 * (r >> 1) + o + (r & 1).  Class 0 starts at the placeholder
// position -1.
__device__ __forceinline__ int64_t class_pos(int b, int64_t r) {
    return 4 * (r >> 1) + (b - 1) + (r & 1);
}
__device__ __forceinline__ int64_t class_rank(int b, int64_t q) {
    const int64_t d = q - (b - 1);
    return 2 * (d >> 2) + (d & 3);
}
// the class a row's skips walk from node (p, pi): {p - 1, p} when pi = 0, {p, p + 1} when 1
__device__ __forceinline__ int node_class(int64_t p, int pi) { return (int)((p + pi) & 3); }

struct Compressed {
    DevState seed;
    double l1mp;
    int64_t nmaj, nmin;
    int64_t words;   // word budget U (a multiple of 4)
    int64_t ranks;   // ranks per residue class
    uint32_t *skip;  // [U] min(skip, nmin), kNearTie flag
    int64_t *csum;   // [4][ranks] inclusive prefix sums of 1 + skip per class
};

__global__ void skip_kernel(Compressed c) {
    const int64_t blocks = c.words / 4;
    for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < blocks;
         b += (int64_t)gridDim.x * blockDim.x) {
        const uint4 r = philox(ctr_add(c.seed.ctr, (uint64_t)b), c.seed.key);
        uint32_t v[4];
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            bool tie;
            const int64_t g = geometric(lane_of(r, l), c.l1mp, tie);
            // a tie matters only where one of the two candidates lands inside the row
            v[l] = (uint32_t)min(g, c.nmin) | (tie && g <= c.nmin ? kNearTie : 0u);
        }
        reinterpret_cast<uint4 *>(c.skip)[b] = make_uint4(v[0], v[1], v[2], v[3]);
    }
}

__global__ void class_terms_kernel(Compressed c) {
    const int64_t total = 4 * c.ranks;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < total;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int b = (int)(t / c.ranks);
        const int64_t q = class_pos(b, t % c.ranks);
        // past the budget: a term that ends any row, so a walk reaching it has overflowed
        c.csum[t] = q < 0 ? 1 : q >= c.words ? 1 + c.nmin : 1 + (int64_t)(c.skip[q] & kSkipMask);
    }
}

// Rank in class b at which the row starting at word p, whose skips walk class b from rank r0,
// ends (its terminating skip), or -1 if that lies beyond the budget.
__device__ int64_t row_end_rank(const Compressed &c, int64_t p, int b, int64_t r0) {
    const int64_t *C = c.csum + b * c.ranks;
    const int64_t g0 = c.skip[p] & kSkipMask;
    if (g0 >= c.nmin) return r0;
    const int64_t target = C[r0] - g0 + c.nmin;  // first r >= r0 with C[r] >= target
    int64_t lo = r0, hi = r0 + 1, step = 1;
    while (hi < c.ranks && C[hi] < target) {
        lo = hi;
        step <<= 1;
        hi = r0 + step;
    }
    if (hi >= c.ranks) {
        hi = c.ranks - 1;
        if (C[hi] < target) return -1;
    }
    while (hi - lo > 1) {
        const int64_t mid = lo + (hi - lo) / 2;
        if (C[mid] < target) lo = mid;
        else hi = mid;
    }
    return hi;
}

// successor node of every node x = 2p + pi (-1: beyond the budget)
__global__ void successor_kernel(Compressed c, int32_t *J) {
    const int64_t nodes = 2 * c.words;
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < nodes;
         x += (int64_t)gridDim.x * blockDim.x) {
        const int64_t p = x >> 1;
        const int pi = (int)(x & 1);
        const int b = node_class(p, pi);
        const int64_t r0 = class_rank(b, p);
        const int64_t r = row_end_rank(c, p, b, r0);
        int32_t s = -1;
        if (r >= 0) {
            const int64_t q = class_pos(b, r);
            if (q + 1 < c.words) s = (int32_t)(2 * (q + 1) + (pi ^ (int)((r - r0) & 1)));
        }
        J[x] = s;
    }
}

// One pointer-jumping round: nodes whose row index d < step mark J^step(x) as row d + step;
// then (if square) J <- J o J.
__global__ void jump_kernel(const int32_t *__restrict__ Jin, int32_t *__restrict__ Jout,
                            int32_t *rid, int64_t nodes, int64_t step, int64_t nmaj, int square,
                            Status *st) {
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < nodes;
         x += (int64_t)gridDim.x * blockDim.x) {
        // rows marked in this round carry d >= step and are not propagated again
        const int32_t d = rid[x];
        const int32_t y = Jin[x];
        if (d >= 0 && d < step && d + step < nmaj) {
            if (y >= 0) rid[y] = (int32_t)(d + step);
            else st->overflow = 1;
        }
        if (square) Jout[x] = y < 0 ? -1 : Jin[y];
    }
}

__global__ void collect_kernel(const int32_t *__restrict__ rid, int64_t nodes, int32_t *start) {
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < nodes;
         x += (int64_t)gridDim.x * blockDim.x) {
        const int32_t d = rid[x];
        if (d >= 0) start[d] = (int32_t)x;
    }
}

// Row i's nonzero count; near-ties among the skips it uses; words consumed after the last row.
__global__ void row_count_kernel(Compressed c, const int32_t *__restrict__ start, int64_t *cnt,
                                 Status *st) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < c.nmaj;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int32_t x = start[i];
        if (x < 0) {
            st->overflow = 1;
            cnt[i] = 0;
            continue;
        }
        const int64_t p = x >> 1;
        const int pi = x & 1;
        const int b = node_class(p, pi);
        const int64_t r0 = class_rank(b, p);
        int64_t r;
        if (i + 1 < c.nmaj) {
            const int32_t x1 = start[i + 1];
            r = x1 < 0 ? -1 : class_rank(b, (int64_t)(x1 >> 1) - 1);
            if (r >= 0 && (r < r0 || r >= c.ranks || class_pos(b, r) != (int64_t)(x1 >> 1) - 1)) {
                st->broken = 1;
                cnt[i] = 0;
                continue;
            }
        } else {
            r = row_end_rank(c, p, b, r0);
            if (r >= 0) st->consumed = class_pos(b, r) + 1;
        }
        if (r < 0) {
            st->overflow = 1;
            cnt[i] = 0;
            continue;
        }
        cnt[i] = r - r0;
        int64_t ties = 0;
        for (int64_t t = r0; t <= r; ++t) {
            const int64_t q = class_pos(b, t);
            if (q < c.words && (c.skip[q] & kNearTie)) ++ties;
        }
        if (ties) atomicAdd(reinterpret_cast<unsigned long long *>(&st->ambiguous),
                            (unsigned long long)ties);
    }
}

// row of nonzero k: the last i with ptr[i] <= k
__device__ __forceinline__ int64_t row_of(const int64_t *__restrict__ ptr, int64_t nmaj,
                                          int64_t k) {
    int64_t lo = 0, hi = nmaj;  // ptr[lo] <= k < ptr[hi]
    while (hi - lo > 1) {
        const int64_t mid = lo + (hi - lo) / 2;
        if (ptr[mid] <= k) lo = mid;
        else hi = mid;
    }
    return lo;
}

// word position of the skip that created nonzero k, and its minor index
__device__ __forceinline__ int64_t nonzero_skip(const Compressed &c,
                                                const int32_t *__restrict__ start,
                                                const int64_t *__restrict__ ptr, int64_t k,
                                                int64_t *minor) {
    const int64_t i = row_of(ptr, c.nmaj, k);
    const int32_t x = start[i];
    const int64_t p = x >> 1;
    const int b = node_class(p, x & 1);
    const int64_t r0 = class_rank(b, p);
    const int64_t r = r0 + (k - ptr[i]);
    if (minor) {
        const int64_t *C = c.csum + b * c.ranks;
        *minor = (int64_t)(c.skip[p] & kSkipMask) + C[r] - C[r0];
    }
    return class_pos(b, r);
}

template <typename T, typename I>
__global__ void emit_compressed_kernel(Compressed c, const int32_t *__restrict__ start,
                                       const int64_t *__restrict__ ptr, int64_t nnz, T *vals,
                                       I *ptr_out, I *minor_out) {
    const int64_t n = std::max<int64_t>(nnz, c.nmaj + 1);
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        if (k <= c.nmaj) ptr_out[k] = (I)ptr[k];
        if (k >= nnz) continue;
        int64_t minor;
        const int64_t q = nonzero_skip(c, start, ptr, k, &minor);
        // the pair follows the skip of nonzero k - (k mod 2)
        const int64_t qp = (k & 1) ? nonzero_skip(c, start, ptr, k - 1, nullptr) : q;
        float first, second;
        gaussian_pair(c.seed, qp + 1, first, second);
        vals[k] = (T)((k & 1) ? second : first);
        minor_out[k] = (I)minor;
    }
}

// ----------------------------------------------------------------- COO
// Nonzero k's skip word: 0 for k = 0, then 2k + 1 (k odd) or 2k (k even); its value pair
// starts at word 1 + 4 * (k / 2).
__device__ __forceinline__ int64_t coo_skip_word(int64_t k) {
    return k == 0 ? 0 : (k & 1) ? 2 * k + 1 : 2 * k;
}

struct SatAdd {
    int64_t cap;
    __host__ __device__ __forceinline__ int64_t operator()(int64_t a, int64_t b) const {
        const int64_t s = a + b;  // both <= cap < 2^62
        return s < cap ? s : cap;
    }
};

__global__ void coo_skip_kernel(DevState seed, double l1mp, int64_t total, int64_t K,
                                int64_t *inc, uint8_t *tie) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < K;
         k += (int64_t)gridDim.x * blockDim.x) {
        bool t;
        const int64_t g = geometric(stream_word(seed, coo_skip_word(k)), l1mp, t);
        inc[k] = min((k == 0 ? 0 : 1) + g, total);
        tie[k] = t ? 1 : 0;
    }
}

__global__ void coo_count_kernel(const int64_t *__restrict__ pos, int64_t K, int64_t total,
                                 Status *st) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < K;
         k += (int64_t)gridDim.x * blockDim.x)
        if (pos[k] >= total && (k == 0 || pos[k - 1] < total)) st->nnz = k;
}

__global__ void coo_ties_kernel(const uint8_t *__restrict__ tie, Status *st) {
    const int64_t nnz = st->nnz;
    unsigned long long n = 0;
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k <= nnz;
         k += (int64_t)gridDim.x * blockDim.x)
        n += tie[k];
    if (n) atomicAdd(reinterpret_cast<unsigned long long *>(&st->ambiguous), n);
}

template <typename T, typename I>
__global__ void emit_coo_kernel(DevState seed, const int64_t *__restrict__ pos, int64_t nnz,
                                int64_t n, T *vals, I *rows, I *cols) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < nnz;
         k += (int64_t)gridDim.x * blockDim.x) {
        float first, second;
        gaussian_pair(seed, 1 + 4 * (k >> 1), first, second);
        vals[k] = (T)((k & 1) ? second : first);
        rows[k] = (I)(pos[k] / n);
        cols[k] = (I)(pos[k] % n);
    }
}

// ----------------------------------------------------------------- density 1 and empty
// Every entry, major index by major index; entry k's value from the pair at words 2 * (k / 2).
template <typename T, typename I>
__global__ void emit_full_kernel(DevState seed, int fmt, int64_t nmaj, int64_t nmin, T *vals,
                                 I *a, I *b) {
    const int64_t total = nmaj * nmin;
    const int64_t n = std::max<int64_t>(total, nmaj + 1);
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        if (fmt != RBG_COO && k <= nmaj) a[k] = (I)(k * nmin);
        if (k >= total) continue;
        const uint4 r = philox(ctr_add(seed.ctr, (uint64_t)k >> 2), seed.key);
        float first, second;
        if (k & 2) boxmuller(r.z, r.w, first, second);
        else boxmuller(r.x, r.y, first, second);
        vals[k] = (T)((k & 1) ? second : first);
        if (fmt == RBG_COO) {
            a[k] = (I)(k / nmin);
            b[k] = (I)(k % nmin);
        } else {
            b[k] = (I)(k % nmin);
        }
    }
}

template <typename I>
__global__ void zero_kernel(I *a, int64_t n) {
    for (int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        a[k] = 0;
}

const char *fn_name(int fmt) {
    return fmt == RBG_COO ? "random_coo" : fmt == RBG_CSR ? "random_csr" : "random_csc";
}

}  // namespace
}  // namespace rbg

using namespace rbg;

struct rbg_random_sparse_s {
    enum Kind { EMPTY, FULL, COO_GEOM, COMPRESSED_GEOM } kind = EMPTY;
    int fmt = RBG_CSR;
    int64_t m = 0, n = 0, nmaj = 0, nmin = 0;
    DevState seed{};
    int64_t nnz = 0, consumed = 0, ambiguous = 0;
    Compressed comp{};
    // device memory kept for the fill: COO positions, or the compressed path's skips, class
    // sums, row starts and pointers
    void *mem = nullptr;
    cudaStream_t stream = nullptr;  // of the last create / fill call: mem is freed on it
    int64_t *coo_pos = nullptr;
    int32_t *start = nullptr;
    int64_t *ptr = nullptr;
};

namespace {

using Handle = rbg_random_sparse_s;

size_t align_up(size_t x) { return (x + 255) & ~size_t(255); }

// Stream-ordered device memory that outlives the call (the handle's), freed by release().
void *device_alloc(size_t bytes, cudaStream_t s) {
    void *p = nullptr;
    const cudaError_t e = cudaMallocAsync(&p, std::max<size_t>(bytes, 256), s);
    if (e != cudaSuccess) {
        cudaGetLastError();
        fail(RBG_ERROR_ALLOC, "cudaMallocAsync of " + std::to_string(bytes) + " bytes failed");
    }
    return p;
}

void read_status(Status &host, const Status *dev, cudaStream_t s) {
    RBG_CUDA(cudaMemcpyAsync(&host, dev, sizeof(Status), cudaMemcpyDeviceToHost, s));
    RBG_CUDA(cudaStreamSynchronize(s));
}

// COO: candidates until the scan passes m * n; returns false when more are needed.
bool coo_attempt(Handle &h, double l1mp, int64_t K, cudaStream_t s) {
    const int64_t total = h.m * h.n;
    Scratch st(sizeof(Status), s), tie(K, s);
    int64_t *pos = static_cast<int64_t *>(device_alloc(sizeof(int64_t) * K, s));
    h.mem = pos;
    RBG_CUDA(cudaMemsetAsync(st.ptr, 0, sizeof(Status), s));
    RBG_CUDA(cudaMemsetAsync(&st.as<Status>()->nnz, 0xFF, sizeof(int64_t), s));
    coo_skip_kernel<<<ctas(K), kThreads, 0, s>>>(h.seed, l1mp, total, K, pos,
                                                     tie.as<uint8_t>());
    RBG_LAUNCHED();
    size_t tmp_bytes = 0;
    RBG_CUDA(cub::DeviceScan::InclusiveScan(nullptr, tmp_bytes, pos, pos, SatAdd{total}, K, s));
    {
        Scratch tmp(tmp_bytes, s);
        RBG_CUDA(cub::DeviceScan::InclusiveScan(tmp.ptr, tmp_bytes, pos, pos, SatAdd{total}, K,
                                                s));
    }
    coo_count_kernel<<<ctas(K), kThreads, 0, s>>>(pos, K, total, st.as<Status>());
    RBG_LAUNCHED();
    Status hs{};
    read_status(hs, st.as<Status>(), s);
    if (hs.nnz < 0) return false;  // every candidate still inside the matrix
    coo_ties_kernel<<<ctas(hs.nnz + 1), kThreads, 0, s>>>(tie.as<uint8_t>(), st.as<Status>());
    RBG_LAUNCHED();
    read_status(hs, st.as<Status>(), s);
    h.nnz = hs.nnz;
    h.ambiguous = hs.ambiguous;
    h.coo_pos = pos;
    // the loop's last draw is the skip that left the matrix
    h.consumed = h.nnz == 0 ? 1 : ((h.nnz & 1) ? 2 * h.nnz + 1 : 2 * h.nnz) + 1;
    return true;
}

// CSR / CSC with a word budget of U; returns false when the rows need more words.
bool compressed_attempt(Handle &h, double l1mp, int64_t U, cudaStream_t s) {
    Compressed c{};
    c.seed = h.seed;
    c.l1mp = l1mp;
    c.nmaj = h.nmaj;
    c.nmin = h.nmin;
    c.words = U;
    c.ranks = U / 2 + 4;
    const int64_t nodes = 2 * U;
    // kept: skips, class sums, row starts, pointers
    const size_t b_skip = align_up(sizeof(uint32_t) * U);
    const size_t b_csum = align_up(sizeof(int64_t) * 4 * c.ranks);
    const size_t b_start = align_up(sizeof(int32_t) * h.nmaj);
    const size_t b_ptr = align_up(sizeof(int64_t) * (h.nmaj + 1));
    char *mem = static_cast<char *>(device_alloc(b_skip + b_csum + b_start + b_ptr, s));
    h.mem = mem;
    c.skip = reinterpret_cast<uint32_t *>(mem);
    c.csum = reinterpret_cast<int64_t *>(mem + b_skip);
    int32_t *start = reinterpret_cast<int32_t *>(mem + b_skip + b_csum);
    int64_t *ptr = reinterpret_cast<int64_t *>(mem + b_skip + b_csum + b_start);

    skip_kernel<<<ctas(U / 4), kThreads, 0, s>>>(c);
    RBG_LAUNCHED();
    class_terms_kernel<<<ctas(4 * c.ranks), kThreads, 0, s>>>(c);
    RBG_LAUNCHED();
    size_t tmp_bytes = 0;
    RBG_CUDA(cub::DeviceScan::InclusiveSum(nullptr, tmp_bytes, c.csum, c.csum, 4 * c.ranks, s));
    {
        Scratch tmp(tmp_bytes, s);
        RBG_CUDA(cub::DeviceScan::InclusiveSum(tmp.ptr, tmp_bytes, c.csum, c.csum, 4 * c.ranks,
                                               s));
    }
    Scratch st(sizeof(Status), s), Ja(sizeof(int32_t) * nodes, s), Jb(sizeof(int32_t) * nodes, s),
        rid(sizeof(int32_t) * nodes, s);
    RBG_CUDA(cudaMemsetAsync(st.ptr, 0, sizeof(Status), s));
    RBG_CUDA(cudaMemsetAsync(rid.ptr, 0xFF, sizeof(int32_t) * nodes, s));
    RBG_CUDA(cudaMemsetAsync(rid.ptr, 0, sizeof(int32_t), s));  // node (0, even) is row 0
    RBG_CUDA(cudaMemsetAsync(start, 0xFF, sizeof(int32_t) * h.nmaj, s));
    successor_kernel<<<ctas(nodes), kThreads, 0, s>>>(c, Ja.as<int32_t>());
    RBG_LAUNCHED();
    int32_t *Jin = Ja.as<int32_t>(), *Jout = Jb.as<int32_t>();
    for (int64_t step = 1; step < h.nmaj; step <<= 1) {
        const int square = 2 * step < h.nmaj;
        jump_kernel<<<ctas(nodes), kThreads, 0, s>>>(Jin, Jout, rid.as<int32_t>(), nodes, step,
                                                         h.nmaj, square, st.as<Status>());
        RBG_LAUNCHED();
        std::swap(Jin, Jout);
    }
    collect_kernel<<<ctas(nodes), kThreads, 0, s>>>(rid.as<int32_t>(), nodes, start);
    RBG_LAUNCHED();
    Scratch cnt(sizeof(int64_t) * (h.nmaj + 1), s);
    RBG_CUDA(cudaMemsetAsync(cnt.as<int64_t>() + h.nmaj, 0, sizeof(int64_t), s));
    row_count_kernel<<<ctas(h.nmaj), kThreads, 0, s>>>(c, start, cnt.as<int64_t>(),
                                                           st.as<Status>());
    RBG_LAUNCHED();
    RBG_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, cnt.as<int64_t>(), ptr,
                                           h.nmaj + 1, s));
    {
        Scratch tmp(tmp_bytes, s);
        RBG_CUDA(cub::DeviceScan::ExclusiveSum(tmp.ptr, tmp_bytes, cnt.as<int64_t>(), ptr,
                                               h.nmaj + 1, s));
    }
    // the pointer array's last entry (nnz) travels back with the status: one read, one sync
    RBG_CUDA(cudaMemcpyAsync(&st.as<Status>()->nnz, ptr + h.nmaj, sizeof(int64_t),
                             cudaMemcpyDeviceToDevice, s));
    Status hs{};
    read_status(hs, st.as<Status>(), s);
    if (hs.broken) fail(RBG_ERROR_CUDA, "random sparse generator: inconsistent row chain");
    if (hs.overflow) return false;
    h.nnz = hs.nnz;
    h.consumed = hs.consumed;
    h.ambiguous = hs.ambiguous;
    h.comp = c;
    h.start = start;
    h.ptr = ptr;
    return true;
}

// Frees the handle's memory in stream order on the stream of its last create / fill call, so
// no sync is needed and work already queued there finishes first.
void release(Handle &h) {
    if (h.mem) cudaFreeAsync(h.mem, h.stream);
    h.mem = nullptr;
}

void create(int32_t fmt, int64_t m, int64_t n, double density, const rbg_state *seed,
            Handle &h, cudaStream_t s) {
    if (fmt != RBG_COO && fmt != RBG_CSR && fmt != RBG_CSC)
        fail(RBG_ERROR_INVALID_ARGUMENT, "format must be RBG_COO, RBG_CSR or RBG_CSC");
    if (!seed) fail(RBG_ERROR_INVALID_ARGUMENT, "seed must not be NULL");
    const char *fn = fn_name(fmt);
    RBG_REQUIRE(fn, density >= 0.0 && density <= 1.0);  // random_matrix.hh:142, 224, 303
    RBG_REQUIRE(fn, m >= 0 && n >= 0);
    h.stream = s;
    h.fmt = fmt;
    h.m = m;
    h.n = n;
    h.nmaj = fmt == RBG_CSC ? n : m;
    h.nmin = fmt == RBG_CSC ? m : n;
    h.seed = to_dev(*seed);
    if (density == 0.0 || m == 0 || n == 0) {
        h.kind = Handle::EMPTY;
        return;
    }
    const int64_t total = safe_mul(m, n);
    if (density >= 1.0) {
        h.kind = Handle::FULL;
        h.nnz = total;
        h.consumed = total + (total & 1);
        return;
    }
    const double l1mp = std::log(1.0 - density);
    if (l1mp == 0.0)
        fail(RBG_ERROR_UNSUPPORTED,
             std::string(fn) + ": log(1 - density) rounds to 0 for density " +
                 std::to_string(density) + "; the reference's skip is then undefined");
    const double mu = (double)total * density, sd = std::sqrt(mu) + 1.0;
    if (fmt == RBG_COO) {
        if (total >= (int64_t(1) << 62))
            fail(RBG_ERROR_UNSUPPORTED, "random_coo: m * n must be below 2^62");
        h.kind = Handle::COO_GEOM;
        // nnz <= m * n, so m * n + 1 candidates always reach the end
        int64_t K = std::min<int64_t>((int64_t)(mu + 8.0 * sd) + 64, total + 1);
        for (;;) {
            if (coo_attempt(h, l1mp, K, s)) return;
            release(h);
            if (K == total + 1) fail(RBG_ERROR_CUDA, "random_coo: candidates exhausted");
            K = std::min<int64_t>(2 * K, total + 1);
        }
    }
    if (h.nmin >= (int64_t(1) << 31) - 1)
        fail(RBG_ERROR_UNSUPPORTED,
             std::string(fn) + ": the minor dimension must be below 2^31 - 1");
    h.kind = Handle::COMPRESSED_GEOM;
    // words: one terminating skip per row, one skip per nonzero and a pair per two nonzeros
    double est = (double)h.nmaj + 2.0 * (mu + 8.0 * sd) + 1024.0;
    for (;;) {
        if (est > (double)kMaxWords)
            fail(RBG_ERROR_UNSUPPORTED,
                 std::string(fn) + ": more than 2^30 stream words (about 5e8 nonzeros)");
        const int64_t U = ((int64_t)est + 3) & ~int64_t(3);
        if (compressed_attempt(h, l1mp, U, s)) return;
        release(h);
        est *= 2.0;
    }
}

template <typename T, typename I>
void fill_t(const Handle &h, void *vals, void *a, void *b, cudaStream_t s) {
    switch (h.kind) {
    case Handle::EMPTY:
        if (h.fmt != RBG_COO && h.nmaj > 0) {
            zero_kernel<I><<<ctas(h.nmaj + 1), kThreads, 0, s>>>(static_cast<I *>(a),
                                                                    h.nmaj + 1);
            RBG_LAUNCHED();
        }
        return;
    case Handle::FULL:
        emit_full_kernel<T, I><<<ctas(std::max(h.nnz, h.nmaj + 1)), kThreads, 0, s>>>(
            h.seed, h.fmt, h.nmaj, h.nmin, static_cast<T *>(vals), static_cast<I *>(a),
            static_cast<I *>(b));
        RBG_LAUNCHED();
        return;
    case Handle::COO_GEOM:
        if (h.nnz == 0) return;
        emit_coo_kernel<T, I><<<ctas(h.nnz), kThreads, 0, s>>>(
            h.seed, h.coo_pos, h.nnz, h.n, static_cast<T *>(vals), static_cast<I *>(a),
            static_cast<I *>(b));
        RBG_LAUNCHED();
        return;
    case Handle::COMPRESSED_GEOM:
        emit_compressed_kernel<T, I><<<ctas(std::max(h.nnz, h.nmaj + 1)), kThreads, 0, s>>>(
            h.comp, h.start, h.ptr, h.nnz, static_cast<T *>(vals), static_cast<I *>(a),
            static_cast<I *>(b));
        RBG_LAUNCHED();
        return;
    }
}

}  // namespace

extern "C" int rbg_random_sparse_create(int32_t format, int64_t m, int64_t n, double density,
                                        const rbg_state *seed, rbg_random_sparse *out,
                                        int64_t *nnz, rbg_state *next, rbg_stream_t stream) {
    return guarded([&] {
        if (!out) fail(RBG_ERROR_INVALID_ARGUMENT, "out must not be NULL");
        *out = nullptr;
        Handle *h = new Handle();
        try {
            create(format, m, n, density, seed, *h, as_cuda(stream));
        } catch (...) {
            release(*h);
            delete h;
            throw;
        }
        if (nnz) *nnz = h->nnz;
        if (next) {
            const uint4 c = ctr_add(h->seed.ctr, (uint64_t)((h->consumed + 3) / 4));
            *next = *seed;
            next->counter[0] = c.x;
            next->counter[1] = c.y;
            next->counter[2] = c.z;
            next->counter[3] = c.w;
        }
        *out = h;
    });
}

extern "C" int rbg_random_sparse_fill(rbg_random_sparse h, int32_t dtype, int32_t itype,
                                      void *vals, void *a, void *b, rbg_stream_t stream) {
    return guarded([&] {
        if (!h) fail(RBG_ERROR_INVALID_ARGUMENT, "handle must not be NULL");
        if (dtype != RBG_F32 && dtype != RBG_F64)
            fail(RBG_ERROR_INVALID_ARGUMENT, "dtype must be RBG_F32 or RBG_F64");
        if (itype != RBG_I32 && itype != RBG_I64)
            fail(RBG_ERROR_INVALID_ARGUMENT, "itype must be RBG_I32 or RBG_I64");
        if (h->nnz > 0 && (!vals || !b || (h->fmt == RBG_COO && !a)))
            fail(RBG_ERROR_INVALID_ARGUMENT, "vals and index arrays must not be NULL");
        if (h->fmt != RBG_COO && h->nmaj > 0 && !a)
            fail(RBG_ERROR_INVALID_ARGUMENT, "the pointer array must not be NULL");
        if (itype == RBG_I32 && (h->nnz > INT32_MAX || h->m > INT32_MAX || h->n > INT32_MAX))
            fail(RBG_ERROR_OVERFLOW, "nnz or a dimension does not fit 32-bit indices");
        const cudaStream_t s = as_cuda(stream);
        h->stream = s;
        if (dtype == RBG_F32 && itype == RBG_I32) fill_t<float, int32_t>(*h, vals, a, b, s);
        else if (dtype == RBG_F32) fill_t<float, int64_t>(*h, vals, a, b, s);
        else if (itype == RBG_I32) fill_t<double, int32_t>(*h, vals, a, b, s);
        else fill_t<double, int64_t>(*h, vals, a, b, s);
    });
}

extern "C" int rbg_random_sparse_info(rbg_random_sparse h, int64_t *near_ties,
                                      int64_t *words_drawn) {
    return guarded([&] {
        if (!h) fail(RBG_ERROR_INVALID_ARGUMENT, "handle must not be NULL");
        if (near_ties) *near_ties = h->ambiguous;
        if (words_drawn) *words_drawn = h->consumed;
    });
}

extern "C" int rbg_random_sparse_destroy(rbg_random_sparse h) {
    return guarded([&] {
        if (!h) return;
        if (h->mem) RBG_CUDA(cudaFreeAsync(h->mem, h->stream));
        h->mem = nullptr;
        delete h;
    });
}

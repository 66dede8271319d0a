// sparse_convert.cu -- conversions of sparse data on the GPU, after RandBLAS's
// sparse_data/base.hh:119-220, 278-302 and conversions.hh:49-121: compressed pointers to sorted
// indices and back, the sort state of COO arrays, and sorting COO arrays into CSR or CSC order.
// Each call checks what the reference checks, with its messages, and synchronises `stream`
// (the checks are read back).
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <string>

#include "rbg_internal.h"

namespace rbg {
namespace {

constexpr int kThreads = 256;

// CTAs of kThreads for a grid-stride loop over n items
inline int ctas(int64_t n) { return grid_stride_ctas(n, kThreads); }

// idxs[e] = j for the segment ptr[j] - ptr[0] <= e < ptr[j + 1] - ptr[0] holding e
template <typename P, typename X>
__global__ void expand_kernel(int64_t num_comp, const P *__restrict__ ptr, int64_t total,
                              X *__restrict__ idxs) {
    const int64_t base = (int64_t)ptr[0];
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < total;
         e += (int64_t)gridDim.x * blockDim.x) {
        int64_t lo = 0, hi = num_comp;  // last j with ptr[j] - base <= e
        while (hi - lo > 1) {
            const int64_t mid = lo + (hi - lo) / 2;
            if ((int64_t)ptr[mid] - base <= e) lo = mid;
            else hi = mid;
        }
        idxs[e] = (X)lo;
    }
}

// flag[0] = 1 if some segment ptr[j + 1] - ptr[j] is negative
template <typename P>
__global__ void segments_kernel(int64_t num_comp, const P *__restrict__ ptr, int *flag) {
    for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < num_comp;
         j += (int64_t)gridDim.x * blockDim.x)
        if (ptr[j + 1] < ptr[j]) flag[0] = 1;
}

// flag[0] = 1 if idxs is not sorted
template <typename X>
__global__ void sorted_kernel(int64_t len, const X *__restrict__ idxs, int *flag) {
    for (int64_t i = 1 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < len;
         i += (int64_t)gridDim.x * blockDim.x)
        if (idxs[i - 1] > idxs[i]) flag[0] = 1;
}

// The reference's walk over sorted idxs: ptr[0] = 0, ptr[i + 1] = #(idxs <= i), except that a
// negative first index stops the walk at 0.
template <typename X, typename P>
__global__ void compress_kernel(int64_t len, const X *__restrict__ idxs, int64_t num_comp,
                                P *__restrict__ ptr) {
    const bool stuck = len > 0 && (int64_t)idxs[0] < 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i <= num_comp;
         i += (int64_t)gridDim.x * blockDim.x) {
        if (i == 0 || stuck) {
            ptr[i] = (P)0;
            continue;
        }
        int64_t lo = 0, hi = len;  // first position with idxs > i - 1
        while (lo < hi) {
            const int64_t mid = lo + (hi - lo) / 2;
            if ((int64_t)idxs[mid] <= i - 1) lo = mid + 1;
            else hi = mid;
        }
        ptr[i] = (P)lo;
    }
}

// flags[0] = 1 if some neighbours are out of CSC order, flags[1] = 1 if out of CSR order
// (increasing_by_csc / increasing_by_csr, sparse_data/base.hh:119-140: ties allowed)
template <typename I>
__global__ void sort_state_kernel(int64_t nnz, const I *__restrict__ rows,
                                  const I *__restrict__ cols, int *flags) {
    for (int64_t e = 1 + blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < nnz;
         e += (int64_t)gridDim.x * blockDim.x) {
        const int64_t i0 = rows[e - 1], j0 = cols[e - 1], i1 = rows[e], j1 = cols[e];
        if (!(j0 < j1 || (j0 == j1 && i0 <= i1))) flags[0] = 1;
        if (!(i0 < i1 || (i0 == i1 && j0 <= j1))) flags[1] = 1;
    }
}

__global__ void iota_kernel64(int64_t n, int64_t *out) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
         e += (int64_t)gridDim.x * blockDim.x)
        out[e] = e;
}

template <typename V>
__global__ void gather_kernel(int64_t n, const int64_t *__restrict__ perm,
                              const V *__restrict__ in, V *__restrict__ out) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n;
         e += (int64_t)gridDim.x * blockDim.x)
        out[e] = in[perm[e]];
}

int read_flag(const Scratch &f, cudaStream_t s) {
    int h = 0;
    RBG_CUDA(cudaMemcpyAsync(&h, f.ptr, sizeof(int), cudaMemcpyDeviceToHost, s));
    RBG_CUDA(cudaStreamSynchronize(s));
    return h;
}

void check_itype_arg(int32_t itype, const char *what) {
    if (itype != RBG_I32 && itype != RBG_I64)
        fail(RBG_ERROR_INVALID_ARGUMENT, std::string(what) + " must be RBG_I32 or RBG_I64");
}

template <typename F>
void by_itype(int32_t itype, F &&f) {
    if (itype == RBG_I32) f(int32_t{});
    else f(int64_t{});
}

int64_t read_index(int32_t itype, const void *p, int64_t i, cudaStream_t s) {
    int64_t v = 0;
    if (itype == RBG_I32) {
        int32_t t = 0;
        RBG_CUDA(cudaMemcpyAsync(&t, static_cast<const int32_t *>(p) + i, sizeof t,
                                 cudaMemcpyDeviceToHost, s));
        RBG_CUDA(cudaStreamSynchronize(s));
        v = t;
    } else {
        RBG_CUDA(cudaMemcpyAsync(&v, static_cast<const int64_t *>(p) + i, sizeof v,
                                 cudaMemcpyDeviceToHost, s));
        RBG_CUDA(cudaStreamSynchronize(s));
    }
    return v;
}

// 'C', 'R' or 'N' (coo_arrays_determine_sort, sparse_data/base.hh:142-167)
int determine_sort(int32_t itype, int64_t nnz, const void *rows, const void *cols,
                   cudaStream_t s) {
    if (nnz <= 1) return RBG_SORT_CSC;
    Scratch flags(2 * sizeof(int), s);
    RBG_CUDA(cudaMemsetAsync(flags.ptr, 0, 2 * sizeof(int), s));
    by_itype(itype, [&](auto tag) {
        using I = decltype(tag);
        sort_state_kernel<I><<<ctas(nnz), kThreads, 0, s>>>(
            nnz, static_cast<const I *>(rows), static_cast<const I *>(cols), flags.as<int>());
        RBG_LAUNCHED();
    });
    int h[2] = {0, 0};
    RBG_CUDA(cudaMemcpyAsync(h, flags.ptr, sizeof h, cudaMemcpyDeviceToHost, s));
    RBG_CUDA(cudaStreamSynchronize(s));
    return !h[0] ? RBG_SORT_CSC : !h[1] ? RBG_SORT_CSR : RBG_SORT_NONE;
}

template <typename K>
void sort_pairs(const K *keys_in, K *keys_out, const int64_t *vals_in, int64_t *vals_out,
                int64_t n, cudaStream_t s) {
    size_t bytes = 0;
    RBG_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, bytes, keys_in, keys_out, vals_in,
                                             vals_out, n, 0, (int)(8 * sizeof(K)), s));
    Scratch tmp(bytes, s);
    RBG_CUDA(cub::DeviceRadixSort::SortPairs(tmp.ptr, bytes, keys_in, keys_out, vals_in,
                                             vals_out, n, 0, (int)(8 * sizeof(K)), s));
}

// Stable sort of (vals, rows, cols) by (major, minor): two stable radix passes, minor first.
template <typename T, typename I>
void apply_sort_t(int32_t sort, int64_t nnz, T *vals, I *rows, I *cols, cudaStream_t s) {
    const I *major = sort == RBG_SORT_CSR ? rows : cols;
    const I *minor = sort == RBG_SORT_CSR ? cols : rows;
    Scratch perm_a(sizeof(int64_t) * nnz, s), perm_b(sizeof(int64_t) * nnz, s),
        keys_a(sizeof(I) * nnz, s), keys_b(sizeof(I) * nnz, s);
    iota_kernel64<<<ctas(nnz), kThreads, 0, s>>>(nnz, perm_a.as<int64_t>());
    RBG_LAUNCHED();
    sort_pairs<I>(minor, keys_b.as<I>(), perm_a.as<int64_t>(), perm_b.as<int64_t>(), nnz, s);
    gather_kernel<I><<<ctas(nnz), kThreads, 0, s>>>(nnz, perm_b.as<int64_t>(), major,
                                                         keys_a.as<I>());
    RBG_LAUNCHED();
    sort_pairs<I>(keys_a.as<I>(), keys_b.as<I>(), perm_b.as<int64_t>(), perm_a.as<int64_t>(),
                  nnz, s);
    const int64_t *perm = perm_a.as<int64_t>();
    Scratch tv(sizeof(T) * nnz, s), ti(sizeof(I) * nnz, s);
    gather_kernel<T><<<ctas(nnz), kThreads, 0, s>>>(nnz, perm, vals, tv.as<T>());
    RBG_LAUNCHED();
    RBG_CUDA(cudaMemcpyAsync(vals, tv.ptr, sizeof(T) * nnz, cudaMemcpyDeviceToDevice, s));
    gather_kernel<I><<<ctas(nnz), kThreads, 0, s>>>(nnz, perm, rows, ti.as<I>());
    RBG_LAUNCHED();
    RBG_CUDA(cudaMemcpyAsync(rows, ti.ptr, sizeof(I) * nnz, cudaMemcpyDeviceToDevice, s));
    gather_kernel<I><<<ctas(nnz), kThreads, 0, s>>>(nnz, perm, cols, ti.as<I>());
    RBG_LAUNCHED();
    RBG_CUDA(cudaMemcpyAsync(cols, ti.ptr, sizeof(I) * nnz, cudaMemcpyDeviceToDevice, s));
    RBG_CUDA(cudaStreamSynchronize(s));
}

void check_ptr(const void *p, const char *what) {
    if (!p) fail(RBG_ERROR_INVALID_ARGUMENT, std::string(what) + " must not be NULL");
}

}  // namespace
}  // namespace rbg

using namespace rbg;

extern "C" int rbg_compressed_ptr_to_sorted_idxs(int64_t num_comp, int32_t ptr_itype,
                                                 const void *ptr, int64_t len_idxs,
                                                 int32_t idx_itype, void *idxs,
                                                 rbg_stream_t stream) {
    return guarded([&] {
        check_itype_arg(ptr_itype, "ptr_itype");
        check_itype_arg(idx_itype, "idx_itype");
        RBG_REQUIRE("compressed_ptr_to_sorted_idxs", num_comp >= 0 && len_idxs >= 0);
        check_ptr(ptr, "ptr");
        const cudaStream_t s = as_cuda(stream);
        const int64_t last = read_index(ptr_itype, ptr, num_comp, s);
        require_as(len_idxs >= last, "len_idxs >= ptr[num_comp]", "compressed_ptr_to_sorted_idxs");
        if (num_comp == 0) return;
        Scratch flag(sizeof(int), s);
        RBG_CUDA(cudaMemsetAsync(flag.ptr, 0, sizeof(int), s));
        by_itype(ptr_itype, [&](auto tag) {
            using P = decltype(tag);
            segments_kernel<P><<<ctas(num_comp), kThreads, 0, s>>>(
                num_comp, static_cast<const P *>(ptr), flag.as<int>());
            RBG_LAUNCHED();
        });
        require_as(!read_flag(flag, s), "col_nnz >= 0", "compressed_ptr_to_sorted_idxs");
        const int64_t total = last - read_index(ptr_itype, ptr, 0, s);
        if (total <= 0) return;
        // a negative ptr[0] would make the reference write past idxs
        if (total > len_idxs)
            fail(RBG_ERROR_INVALID_ARGUMENT,
                 "compressed_ptr_to_sorted_idxs: ptr[num_comp] - ptr[0] exceeds len_idxs");
        check_ptr(idxs, "idxs");
        by_itype(ptr_itype, [&](auto ptag) {
            using P = decltype(ptag);
            by_itype(idx_itype, [&](auto xtag) {
                using X = decltype(xtag);
                expand_kernel<P, X><<<ctas(total), kThreads, 0, s>>>(
                    num_comp, static_cast<const P *>(ptr), total, static_cast<X *>(idxs));
                RBG_LAUNCHED();
            });
        });
        RBG_CUDA(cudaStreamSynchronize(s));
    });
}

extern "C" int rbg_sorted_idxs_to_compressed_ptr(int64_t len_idxs, int32_t idx_itype,
                                                 const void *idxs, int64_t num_comp,
                                                 int32_t ptr_itype, void *ptr,
                                                 rbg_stream_t stream) {
    return guarded([&] {
        check_itype_arg(ptr_itype, "ptr_itype");
        check_itype_arg(idx_itype, "idx_itype");
        RBG_REQUIRE("sorted_idxs_to_compressed_ptr", num_comp >= 0 && len_idxs >= 0);
        check_ptr(ptr, "ptr");
        if (len_idxs > 0) check_ptr(idxs, "idxs");
        const cudaStream_t s = as_cuda(stream);
        if (len_idxs > 1) {
            Scratch flag(sizeof(int), s);
            RBG_CUDA(cudaMemsetAsync(flag.ptr, 0, sizeof(int), s));
            by_itype(idx_itype, [&](auto tag) {
                using X = decltype(tag);
                sorted_kernel<X><<<ctas(len_idxs), kThreads, 0, s>>>(
                    len_idxs, static_cast<const X *>(idxs), flag.as<int>());
                RBG_LAUNCHED();
            });
            require_as(!read_flag(flag, s), "idxs[i - 1] <= idxs[i]",
                       "sorted_idxs_to_compressed_ptr");
        }
        by_itype(idx_itype, [&](auto xtag) {
            using X = decltype(xtag);
            by_itype(ptr_itype, [&](auto ptag) {
                using P = decltype(ptag);
                compress_kernel<X, P><<<ctas(num_comp + 1), kThreads, 0, s>>>(
                    len_idxs, static_cast<const X *>(idxs), num_comp, static_cast<P *>(ptr));
                RBG_LAUNCHED();
            });
        });
        RBG_CUDA(cudaStreamSynchronize(s));
    });
}

extern "C" int rbg_coo_determine_sort(int32_t itype, int64_t nnz, const void *rows,
                                      const void *cols, int32_t *sort, rbg_stream_t stream) {
    return guarded([&] {
        check_itype_arg(itype, "itype");
        check_ptr(sort, "sort");
        RBG_REQUIRE("coo_arrays_determine_sort", nnz >= 0);
        if (nnz > 1) {
            check_ptr(rows, "rows");
            check_ptr(cols, "cols");
        }
        *sort = determine_sort(itype, nnz, rows, cols, as_cuda(stream));
    });
}

extern "C" int rbg_coo_apply_sort(int32_t sort, int32_t dtype, int32_t itype, int64_t nnz,
                                  void *vals, void *rows, void *cols, rbg_stream_t stream) {
    return guarded([&] {
        if (sort != RBG_SORT_CSC && sort != RBG_SORT_CSR && sort != RBG_SORT_NONE)
            fail(RBG_ERROR_INVALID_ARGUMENT, "sort must be RBG_SORT_CSC, RBG_SORT_CSR or "
                                             "RBG_SORT_NONE");
        if (dtype != RBG_F32 && dtype != RBG_F64)
            fail(RBG_ERROR_INVALID_ARGUMENT, "dtype must be RBG_F32 or RBG_F64");
        check_itype_arg(itype, "itype");
        RBG_REQUIRE("coo_arrays_apply_sort", nnz >= 0);
        if (sort == RBG_SORT_NONE || nnz <= 1) return;
        check_ptr(vals, "vals");
        check_ptr(rows, "rows");
        check_ptr(cols, "cols");
        const cudaStream_t s = as_cuda(stream);
        if (determine_sort(itype, nnz, rows, cols, s) == sort) return;
        by_itype(itype, [&](auto tag) {
            using I = decltype(tag);
            if (dtype == RBG_F32)
                apply_sort_t<float, I>(sort, nnz, static_cast<float *>(vals),
                                       static_cast<I *>(rows), static_cast<I *>(cols), s);
            else
                apply_sort_t<double, I>(sort, nnz, static_cast<double *>(vals),
                                        static_cast<I *>(rows), static_cast<I *>(cols), s);
        });
    });
}

/*
 * oracle.c -- CPU restatement of RandBLAS's sketching hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle the CUDA library in
 * randblas_gb300/ is tested against.  Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU baseline leg may load it; the product never links, calls or falls
 * back to it.
 *
 * Everything here is written from the reference's documented behaviour, one
 * function per reference routine, each citing the reference file:line it
 * restates (paths are relative to the RandBLAS source tree):
 *
 *   Philox4x32-10 ............ Random123 r123::Philox4x32 (used at RandBLAS/base.hh:53).
 *                              Random123 is a third-party dependency that the reference
 *                              does not vendor (CI clones HEAD, unpinned); the bijection is
 *                              restated from its published description: Salmon, Moraes,
 *                              Dror, Shaw, "Parallel Random Numbers: As Easy as 1, 2, 3",
 *                              SC'11, section 4 (Philox-4x32 with R = 10 rounds).
 *                              Pinned by test/test_basic_rng/r123_kat_vectors.txt:19-21.
 *   128-bit counter increment  Random123 r123array4x32::incr(uint64), asserted by
 *                              test/test_basic_rng/test_r123.cc:705-797.
 *   uneg11 / u01 / boxmuller . Random123 uniform.hpp / boxmuller.hpp, as used by
 *                              RandBLAS/random_gen.hh:60-137 (documented definitions:
 *                              u01(x) = x*2^-32 + 2^-33, uneg11(x) = (int32)x*2^-31 + 2^-32,
 *                              boxmuller = (sin(pi*uneg11(u0))*r, cos(pi*uneg11(u0))*r),
 *                              r = sqrt(-2 log u01(u1))).  sin / cos / log come from the
 *                              host libm by default (as in the reference), or, in the
 *                              "shared math" mode (orc_set_math(1)), from shared_math.cc.
 *   fill_dense_submat ........ RandBLAS/dense_skops.hh:96-170
 *   fill_dense_unpacked ...... RandBLAS/dense_skops.hh:563-606
 *   dense compute_next_state . RandBLAS/dense_skops.hh:172-185
 *   natural_layout ........... RandBLAS/dense_skops.hh:187-199
 *   repeated_fisher_yates .... RandBLAS/sparse_skops.hh:51-106
 *   sample_indices_iid_uniform RandBLAS/util.hh:516-546
 *   laso merge ............... RandBLAS/sparse_skops.hh:453-491 (duplicates merged to
 *                              sqrt(count) * first sign; emitted in first-occurrence
 *                              order -- the reference emits them in std::unordered_map
 *                              order, which is implementation-defined, so only the set
 *                              of (index, value) pairs per vector is comparable)
 *   sparse compute_next_state  RandBLAS/sparse_skops.hh:266-283
 *   PhiloxStream, random_csr/csc/coo
 *                              RandBLAS/sparse_data/random_matrix.hh:63-121, 135-355
 *   compressed_ptr_to_sorted_idxs, sorted_idxs_to_compressed_ptr, coo_arrays_determine_sort,
 *   coo_arrays_apply_sort .... RandBLAS/sparse_data/base.hh:119-220, 278-302
 *
 * Build: gcc -O2 -std=gnu11 -fPIC -ffp-contract=off -fopenmp, linked with shared_math.cc
 * (oracle/build.py).
 */
#define _GNU_SOURCE 1 /* sincosf */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_COL_MAJOR 0
#define ORC_ROW_MAJOR 1
#define ORC_GAUSSIAN 0
#define ORC_UNIFORM 1
#define ORC_AXIS_SHORT 0
#define ORC_AXIS_LONG 1
#define ORC_F32 0
#define ORC_F64 1
#define ORC_I32 0
#define ORC_I64 1

typedef struct {
    uint32_t counter[4];
    uint32_t key[2];
} orc_state;

/* ---------------------------------------------------------------- Philox */

/* Round multipliers and Weyl key increments of Philox-4x32 (SC'11, table 2 / sec. 4). */
static const uint32_t kPhiloxMulA = 0xD2511F53u;
static const uint32_t kPhiloxMulB = 0xCD9E8D57u;
static const uint32_t kPhiloxWeylA = 0x9E3779B9u;
static const uint32_t kPhiloxWeylB = 0xBB67AE85u;

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t x0 = ctr[0], x1 = ctr[1], x2 = ctr[2], x3 = ctr[3];
    uint32_t ka = key[0], kb = key[1];
    for (int round = 0; round < 10; ++round) {
        if (round > 0) {
            ka += kPhiloxWeylA;
            kb += kPhiloxWeylB;
        }
        uint64_t pa = (uint64_t)kPhiloxMulA * x0;
        uint64_t pb = (uint64_t)kPhiloxMulB * x2;
        uint32_t n0 = (uint32_t)(pb >> 32) ^ x1 ^ ka;
        uint32_t n1 = (uint32_t)pb;
        uint32_t n2 = (uint32_t)(pa >> 32) ^ x3 ^ kb;
        uint32_t n3 = (uint32_t)pa;
        x0 = n0; x1 = n1; x2 = n2; x3 = n3;
    }
    out[0] = x0; out[1] = x1; out[2] = x2; out[3] = x3;
}

/* counter <- counter + n, the counter read as a little-endian 128-bit integer. */
void orc_ctr_add(uint32_t c[4], uint64_t n) {
    uint64_t t = (uint64_t)c[0] + (n & 0xFFFFFFFFu);
    c[0] = (uint32_t)t;
    t = (uint64_t)c[1] + (n >> 32) + (t >> 32);
    c[1] = (uint32_t)t;
    t = (uint64_t)c[2] + (t >> 32);
    c[2] = (uint32_t)t;
    c[3] += (uint32_t)(t >> 32);
}

/* key <- key + k, the key read as a little-endian 64-bit integer (RNGState(k), base.hh:119). */
void orc_key_from_u64(uint64_t k, uint32_t key[2]) {
    key[0] = (uint32_t)k;
    key[1] = (uint32_t)(k >> 32);
}

/* ------------------------------------------------------------ transforms */

float orc_uneg11(uint32_t u) { return (float)(int32_t)u * 0x1p-31f + 0x1p-32f; }

float orc_u01(uint32_t u) { return (float)u * 0x1p-32f + 0x1p-33f; }

/* Math functions of the Box-Muller transform: 0 = the host libm (glibc's sincosf / logf, as
 * the reference calls them), 1 = the shared specification of shared_math.cc (the same
 * float-float functions the GPU evaluates), for bit-for-bit comparisons. */
static int g_math_mode = 0;
void orc_ffm_sincosf(float theta, float *s, float *c);
float orc_ffm_logf(float x);

void orc_set_math(int mode) { g_math_mode = mode; }
int orc_get_math(void) { return g_math_mode; }

void orc_boxmuller(uint32_t u0, uint32_t u1, float *first, float *second) {
    float s, c, l;
    const float theta = 3.14159265358979323846f * orc_uneg11(u0);
    if (g_math_mode == 1) {
        orc_ffm_sincosf(theta, &s, &c);
        l = orc_ffm_logf(orc_u01(u1));
    } else {
        sincosf(theta, &s, &c);
        l = logf(orc_u01(u1));
    }
    float r = sqrtf(-2.0f * l);
    *first = s * r;
    *second = c * r;
}

/* The four floats one Philox call yields for a dense operator (random_gen.hh:85-137). */
static void gen4(int family, const uint32_t ctr[4], const uint32_t key[2], float v[4]) {
    uint32_t r[4];
    orc_philox4x32_10(ctr, key, r);
    if (family == ORC_GAUSSIAN) {
        orc_boxmuller(r[0], r[1], &v[0], &v[1]);
        orc_boxmuller(r[2], r[3], &v[2], &v[3]);
    } else {
        for (int l = 0; l < 4; ++l) v[l] = orc_uneg11(r[l]);
    }
}

/* ----------------------------------------------------------- dense fills */

int orc_natural_layout(int major_axis, int64_t n_rows, int64_t n_cols) {
    int wide = n_rows < n_cols;
    int is_long = major_axis == ORC_AXIS_LONG;
    if (wide) return is_long ? ORC_ROW_MAJOR : ORC_COL_MAJOR;
    return is_long ? ORC_COL_MAJOR : ORC_ROW_MAJOR;
}

int64_t orc_dim_major(int major_axis, int64_t n_rows, int64_t n_cols) {
    int64_t mx = n_rows > n_cols ? n_rows : n_cols;
    int64_t mn = n_rows > n_cols ? n_cols : n_rows;
    return major_axis == ORC_AXIS_LONG ? mx : mn;
}

/*
 * Row-major n_srows x n_scols block of the implicit row-major parent with n_cols
 * columns, starting at linear offset ptr.  Row R of the parent owns counters
 * [R*ceil(n_cols/4), (R+1)*ceil(n_cols/4)); column C sits in lane C%4 of counter C/4
 * of its row.  Returns seed + (first counter used) + n_srows*ceil(n_cols/4)
 * (dense_skops.hh:96-170).  No scaling, promotes float -> T.
 */
void orc_fill_dense_submat(int dtype, int family, int64_t n_cols, void *smat, int64_t n_srows,
                           int64_t n_scols, int64_t ptr, const orc_state *seed, int64_t lda,
                           orc_state *next) {
    if (lda <= 0) lda = n_scols;
    const int64_t stride = (n_cols + 3) / 4;
    const int64_t r0 = ptr / n_cols, c0 = ptr % n_cols;
    const int64_t blk_first = c0 / 4, blk_last = (c0 + n_scols - 1) / 4;
#pragma omp parallel for schedule(static)
    for (int64_t r = 0; r < n_srows; ++r) {
        uint32_t row_ctr[4];
        memcpy(row_ctr, seed->counter, sizeof row_ctr);
        orc_ctr_add(row_ctr, (uint64_t)((r0 + r) * stride));
        for (int64_t blk = blk_first; blk <= blk_last; ++blk) {
            uint32_t c[4];
            memcpy(c, row_ctr, sizeof c);
            orc_ctr_add(c, (uint64_t)blk);
            float v[4];
            gen4(family, c, seed->key, v);
            for (int l = 0; l < 4; ++l) {
                int64_t col = blk * 4 + l - c0;
                if (col < 0 || col >= n_scols) continue;
                if (dtype == ORC_F32)
                    ((float *)smat)[r * lda + col] = v[l];
                else
                    ((double *)smat)[r * lda + col] = (double)v[l];
            }
        }
    }
    *next = *seed;
    orc_ctr_add(next->counter, (uint64_t)(r0 * stride + blk_first + n_srows * stride));
}

/* dense_skops.hh:563-606: fill an n_rows x n_cols submatrix at (ro_s, co_s) in `layout`. */
int orc_fill_dense_unpacked(int dtype, int layout, int64_t D_rows, int64_t D_cols, int family,
                            int major_axis, int64_t n_rows, int64_t n_cols, int64_t ro_s,
                            int64_t co_s, void *buff, const orc_state *seed, orc_state *next) {
    if (D_rows < n_rows + ro_s || D_cols < n_cols + co_s) return 1;
    const int natural = orc_natural_layout(major_axis, D_rows, D_cols);
    const int64_t ma_len = orc_dim_major(major_axis, D_rows, D_cols);
    int64_t nr, nc, ptr;
    if (natural == ORC_COL_MAJOR) {
        nr = n_cols; nc = n_rows; ptr = ro_s + co_s * ma_len;
    } else {
        nr = n_rows; nc = n_cols; ptr = ro_s * ma_len + co_s;
    }
    orc_fill_dense_submat(dtype, family, ma_len, buff, nr, nc, ptr, seed, 0, next);
    const int64_t size = nr * nc;
    if (family == ORC_UNIFORM) {
        if (dtype == ORC_F32) {
            const float s3 = (float)sqrt(3.0);
            for (int64_t i = 0; i < size; ++i) ((float *)buff)[i] *= s3;
        } else {
            const double s3 = sqrt(3.0);
            for (int64_t i = 0; i < size; ++i) ((double *)buff)[i] *= s3;
        }
    }
    if (layout != natural && size > 0) {
        /* the packed natural-layout block is row-major nr x nc; the other layout is its transpose */
        size_t esz = dtype == ORC_F32 ? 4 : 8;
        char *tmp = (char *)malloc(size * esz);
        if (!tmp) return 2;
        memcpy(tmp, buff, size * esz);
        for (int64_t i = 0; i < nr; ++i)
            for (int64_t j = 0; j < nc; ++j)
                memcpy((char *)buff + (j * nr + i) * esz, tmp + (i * nc + j) * esz, esz);
        free(tmp);
    }
    return 0;
}

/* dense_skops.hh:172-185 */
void orc_dense_next_state(int major_axis, int64_t D_rows, int64_t D_cols, const orc_state *seed,
                          orc_state *next) {
    int64_t ma = orc_dim_major(major_axis, D_rows, D_cols);
    int64_t mi = D_rows + D_cols - ma;
    *next = *seed;
    orc_ctr_add(next->counter, (uint64_t)(((ma + 3) / 4) * mi));
}

/* ---------------------------------------------------------- sparse fills */

static void put_idx(int itype, void *p, int64_t i, int64_t v) {
    if (itype == ORC_I32) ((int32_t *)p)[i] = (int32_t)v;
    else ((int64_t *)p)[i] = v;
}
static void put_val(int dtype, void *p, int64_t i, double v) {
    if (dtype == ORC_F32) ((float *)p)[i] = (float)v;
    else ((double *)p)[i] = v;
}

/*
 * sparse_skops.hh:51-106.  For each minor index i, vec_nnz steps of a Fisher-Yates
 * shuffle of the identity over [0, dim_major); step j of vector i uses counter
 * seed + i*vec_nnz + j, draws ell = j + x0 mod (dim_major - j), and gives a sign from
 * the parity of x1.  The shuffle is undone after each vector, so vectors are independent.
 */
int orc_repeated_fisher_yates(int dtype, int itype, const orc_state *seed, int64_t vec_nnz,
                              int64_t dim_major, int64_t dim_minor, void *idxs_major,
                              void *idxs_minor, void *vals, orc_state *next) {
    if (vec_nnz > dim_major) return 1;
    int64_t *perm = (int64_t *)malloc(sizeof(int64_t) * (size_t)dim_major);
    int64_t *piv = (int64_t *)malloc(sizeof(int64_t) * (size_t)(vec_nnz > 0 ? vec_nnz : 1));
    if (!perm || !piv) { free(perm); free(piv); return 2; }
    for (int64_t t = 0; t < dim_major; ++t) perm[t] = t;
    for (int64_t i = 0; i < dim_minor; ++i) {
        for (int64_t j = 0; j < vec_nnz; ++j) {
            uint32_t c[4], r[4];
            memcpy(c, seed->counter, sizeof c);
            orc_ctr_add(c, (uint64_t)(i * vec_nnz + j));
            orc_philox4x32_10(c, seed->key, r);
            int64_t ell = j + (int64_t)(r[0] % (uint64_t)(dim_major - j));
            piv[j] = ell;
            int64_t picked = perm[ell];
            perm[ell] = perm[j];
            perm[j] = picked;
            put_idx(itype, idxs_major, i * vec_nnz + j, picked);
            if (idxs_minor) put_idx(itype, idxs_minor, i * vec_nnz + j, i);
            if (vals) put_val(dtype, vals, i * vec_nnz + j, (r[1] % 2 == 0) ? 1.0 : -1.0);
        }
        for (int64_t j = vec_nnz - 1; j >= 0; --j) {  /* undo the swaps, last first */
            int64_t ell = piv[j];
            int64_t t = perm[j];
            perm[j] = perm[ell];
            perm[ell] = t;
        }
    }
    free(perm);
    free(piv);
    *next = *seed;
    orc_ctr_add(next->counter, (uint64_t)(dim_minor * vec_nnz));
    return 0;
}

/*
 * util.hh:516-546 with Rademachers.  Sample j of a call uses counter state + j/2,
 * lanes 2*(j%2) (index) and 2*(j%2)+1 (sign); the call consumes ceil(k/2) counters.
 * index = trunc(n * ((double)uneg11(x) + 1) / 2); sign = +1 iff uneg11(x') >= 0.
 */
void orc_sample_indices_iid_uniform(int64_t n, int64_t k, int64_t *samples, double *signs,
                                    const orc_state *state, orc_state *next) {
    for (int64_t j = 0; j < k; ++j) {
        uint32_t c[4], r[4];
        memcpy(c, state->counter, sizeof c);
        orc_ctr_add(c, (uint64_t)(j / 2));
        orc_philox4x32_10(c, state->key, r);
        int lane = 2 * (int)(j % 2);
        double u = ((double)orc_uneg11(r[lane]) + 1.0) / 2.0;
        samples[j] = (int64_t)((double)n * u);
        if (signs) signs[j] = orc_uneg11(r[lane + 1]) >= 0.0f ? 1.0 : -1.0;
    }
    *next = *state;
    orc_ctr_add(next->counter, (uint64_t)((k + 1) / 2));
}

/*
 * LASO fill (sparse_skops.hh:515-565 long-axis branch + merge at :453-491): one
 * long-axis vector per minor index i, vec_nnz iid samples each; duplicates inside a
 * vector merge into one entry of value sqrt(count) * (sign of first occurrence).
 * Writes nnz; returns the state after the last vector.
 */
int orc_fill_laso(int dtype, int itype, int64_t vec_nnz, int64_t dim_major, int64_t dim_minor,
                  void *idxs_long, void *idxs_short, void *vals, int64_t *nnz,
                  const orc_state *seed, orc_state *next) {
    int64_t *smp = (int64_t *)malloc(sizeof(int64_t) * (size_t)vec_nnz);
    double *sg = (double *)malloc(sizeof(double) * (size_t)vec_nnz);
    int64_t *cnt = (int64_t *)malloc(sizeof(int64_t) * (size_t)vec_nnz);
    if (!smp || !sg || !cnt) { free(smp); free(sg); free(cnt); return 2; }
    orc_state st = *seed;
    int64_t total = 0;
    for (int64_t i = 0; i < dim_minor; ++i) {
        orc_state nx;
        orc_sample_indices_iid_uniform(dim_major, vec_nnz, smp, sg, &st, &nx);
        st = nx;
        int64_t distinct = 0;
        for (int64_t j = 0; j < vec_nnz; ++j) {
            int64_t found = -1;
            for (int64_t q = 0; q < distinct; ++q)
                if (smp[q] == smp[j]) { found = q; break; }
            if (found >= 0) {
                cnt[found] += 1;
            } else {
                smp[distinct] = smp[j];
                sg[distinct] = sg[j];
                cnt[distinct] = 1;
                distinct += 1;
            }
        }
        for (int64_t q = 0; q < distinct; ++q) {
            double v;
            if (dtype == ORC_F32) v = (double)(sqrtf((float)cnt[q]) * (float)sg[q]);
            else v = sqrt((double)cnt[q]) * sg[q];
            put_idx(itype, idxs_long, total + q, smp[q]);
            put_idx(itype, idxs_short, total + q, i);
            put_val(dtype, vals, total + q, v);
        }
        total += distinct;
    }
    free(smp);
    free(sg);
    free(cnt);
    *nnz = total;
    *next = st;
    return 0;
}

/* sparse_skops.hh:266-283 */
void orc_sparse_next_state(int major_axis, int64_t D_rows, int64_t D_cols, int64_t vec_nnz,
                           const orc_state *seed, orc_state *next) {
    int64_t mx = D_rows > D_cols ? D_rows : D_cols;
    int64_t mn = D_rows > D_cols ? D_cols : D_rows;
    int64_t incr = major_axis == ORC_AXIS_SHORT ? mx * vec_nnz : mn * ((vec_nnz + 1) / 2);
    *next = *seed;
    orc_ctr_add(next->counter, (uint64_t)incr);
}

/*
 * fill_sparse (sparse_skops.hh:515-565, 587-603): SASO (Axis::Short) or LASO (Axis::Long)
 * into COO arrays (rows, cols, vals) of length >= vec_nnz * dim_minor.  Short-axis indices
 * go to `rows` when n_rows <= n_cols, else to `cols`.  Returns the state after sampling.
 */
int orc_fill_sparse(int dtype, int itype, int64_t D_rows, int64_t D_cols, int64_t vec_nnz,
                    int major_axis, void *vals, void *rows, void *cols, int64_t *nnz,
                    const orc_state *seed, orc_state *next) {
    int64_t mx = D_rows > D_cols ? D_rows : D_cols;
    int64_t mn = D_rows > D_cols ? D_cols : D_rows;
    void *idxs_short = D_rows <= D_cols ? rows : cols;
    void *idxs_long = D_rows <= D_cols ? cols : rows;
    if (major_axis == ORC_AXIS_SHORT) {
        int rc = orc_repeated_fisher_yates(dtype, itype, seed, vec_nnz, mn, mx, idxs_short,
                                           idxs_long, vals, next);
        *nnz = vec_nnz * mx;
        return rc;
    }
    return orc_fill_laso(dtype, itype, vec_nnz, mx, mn, idxs_long, idxs_short, vals, nnz, seed,
                         next);
}

/* ------------------------------------------------ random sparse matrices */

/*
 * PhiloxStream (sparse_data/random_matrix.hh:63-121): 32-bit words dispensed one at a time
 * from the Philox blocks at counters seed, seed + 1, ...; a Gaussian is the first value of
 * boxmuller on a fresh word pair, or the cached second value of the previous pair; a
 * geometric draw is floor(log(1 - u) / log(1 - p)) with u = w * 2^-32 + 2^-33 in double.
 * The state handed back is the counter after the last block fetched.
 */
typedef struct {
    orc_state s;
    uint32_t buf[4];
    int pos;
    float spare;
    int has_spare;
} orc_pstream;

static uint32_t ps_word(orc_pstream *p) {
    if (p->pos >= 4) {
        orc_philox4x32_10(p->s.counter, p->s.key, p->buf);
        orc_ctr_add(p->s.counter, 1);
        p->pos = 0;
    }
    return p->buf[p->pos++];
}

static float ps_gaussian(orc_pstream *p) {
    if (p->has_spare) {
        p->has_spare = 0;
        return p->spare;
    }
    uint32_t a = ps_word(p), b = ps_word(p);
    float g1, g2;
    orc_boxmuller(a, b, &g1, &g2);
    p->spare = g2;
    p->has_spare = 1;
    return g1;
}

static int64_t ps_geometric(orc_pstream *p, double log_1_minus_p) {
    double u = (double)ps_word(p) * 0x1p-32 + 0x1p-33;
    return (int64_t)floor(log(1.0 - u) / log_1_minus_p);
}

/*
 * random_csr / random_csc / random_coo (sparse_data/random_matrix.hh:135-207, 217-285,
 * 296-355).  fmt: 0 = COO (a = rows, b = cols, both of length nnz, CSR order), 1 = CSR
 * (a = rowptr[m + 1], b = colidxs[nnz]), 2 = CSC (a = colptr[n + 1], b = rowidxs[nnz]).
 * Nonzeros past `cap` are drawn but not stored, so a caller can size the arrays from the
 * returned nnz and call again.  Returns nnz, or -1 if density is outside [0, 1] (the
 * reference's randblas_require), or -2 if log(1 - density) rounds to zero (0 < density
 * < 2^-53, where the reference converts an infinite quotient to int64).
 */
int64_t orc_random_sparse(int fmt, int dtype, int itype, int64_t m, int64_t n, double density,
                          const orc_state *seed, int64_t cap, void *vals, void *a, void *b,
                          orc_state *next) {
    if (!(density >= 0.0 && density <= 1.0)) return -1;
    orc_pstream p;
    p.s = *seed;
    p.pos = 4;
    p.spare = 0.0f;
    p.has_spare = 0;
    int64_t k = 0;
    const int compressed = fmt != 0;
    const int64_t nmaj = fmt == 2 ? n : m, nmin = fmt == 2 ? m : n;
    if (density == 0.0 || m == 0 || n == 0) {
        if (compressed)
            for (int64_t i = 0; i <= nmaj && nmaj > 0; ++i) put_idx(itype, a, i, 0);
        *next = p.s;
        return 0;
    }
    if (density >= 1.0) {
        for (int64_t i = 0; i < nmaj; ++i) {
            if (compressed) put_idx(itype, a, i, k);
            for (int64_t j = 0; j < nmin; ++j, ++k) {
                float v = ps_gaussian(&p);
                if (k >= cap) continue;
                put_val(dtype, vals, k, v);
                if (compressed) {
                    put_idx(itype, b, k, j);
                } else {
                    put_idx(itype, a, k, i);
                    put_idx(itype, b, k, j);
                }
            }
        }
        if (compressed) put_idx(itype, a, nmaj, k);
        *next = p.s;
        return k;
    }
    const double l1mp = log(1.0 - density);
    if (l1mp == 0.0) return -2;
    if (compressed) {
        for (int64_t i = 0; i < nmaj; ++i) {
            put_idx(itype, a, i, k);
            int64_t j = ps_geometric(&p, l1mp);
            while (j < nmin) {
                float v = ps_gaussian(&p);
                if (k < cap) {
                    put_val(dtype, vals, k, v);
                    put_idx(itype, b, k, j);
                }
                ++k;
                j += 1 + ps_geometric(&p, l1mp);
            }
        }
        put_idx(itype, a, nmaj, k);
    } else {
        const int64_t total = m * n;
        int64_t pos = ps_geometric(&p, l1mp);
        while (pos < total) {
            float v = ps_gaussian(&p);
            if (k < cap) {
                put_idx(itype, a, k, pos / n);
                put_idx(itype, b, k, pos % n);
                put_val(dtype, vals, k, v);
            }
            ++k;
            pos += 1 + ps_geometric(&p, l1mp);
        }
    }
    *next = p.s;
    return k;
}

/* ------------------------------------------------------ sparse conversions */

static int64_t get_idx(int itype, const void *p, int64_t i) {
    return itype == ORC_I32 ? (int64_t)((const int32_t *)p)[i] : ((const int64_t *)p)[i];
}

/*
 * compressed_ptr_to_sorted_idxs (sparse_data/base.hh:292-302): index j repeated
 * ptr[j + 1] - ptr[j] times, from idxs[0].  Returns 1 if len_idxs < ptr[num_comp], 2 at the
 * first negative segment length (after writing the segments before it), else 0.
 */
int orc_compressed_ptr_to_sorted_idxs(int64_t num_comp, int ptr_itype, const void *ptr,
                                      int64_t len_idxs, int idx_itype, void *idxs) {
    if (len_idxs < get_idx(ptr_itype, ptr, num_comp)) return 1;
    int64_t out = 0;
    for (int64_t j = 0; j < num_comp; ++j) {
        int64_t cnt = get_idx(ptr_itype, ptr, j + 1) - get_idx(ptr_itype, ptr, j);
        if (cnt < 0) return 2;
        for (int64_t t = 0; t < cnt; ++t) put_idx(idx_itype, idxs, out++, j);
    }
    return 0;
}

/*
 * sorted_idxs_to_compressed_ptr (sparse_data/base.hh:278-290): returns 1 if idxs is not
 * sorted; else ptr[0] = 0 and ptr[i + 1] = the position after walking past the entries equal
 * to i, in order.
 */
int orc_sorted_idxs_to_compressed_ptr(int64_t len_idxs, int idx_itype, const void *idxs,
                                      int64_t num_comp, int ptr_itype, void *ptr) {
    for (int64_t i = 1; i < len_idxs; ++i)
        if (get_idx(idx_itype, idxs, i - 1) > get_idx(idx_itype, idxs, i)) return 1;
    put_idx(ptr_itype, ptr, 0, 0);
    int64_t ell = 0;
    for (int64_t i = 0; i < num_comp; ++i) {
        while (ell < len_idxs && get_idx(idx_itype, idxs, ell) == i) ++ell;
        put_idx(ptr_itype, ptr, i + 1, ell);
    }
    return 0;
}

/* coo_arrays_determine_sort (sparse_data/base.hh:119-167): 'C', 'R' or 'N'. */
int orc_coo_determine_sort(int itype, int64_t nnz, const void *rows, const void *cols) {
    int csc = 1, csr = 1;
    for (int64_t e = 1; e < nnz && (csc || csr); ++e) {
        int64_t i0 = get_idx(itype, rows, e - 1), j0 = get_idx(itype, cols, e - 1);
        int64_t i1 = get_idx(itype, rows, e), j1 = get_idx(itype, cols, e);
        if (csc) csc = j0 < j1 || (j0 == j1 && i0 <= i1);
        if (csr) csr = i0 < i1 || (i0 == i1 && j0 <= j1);
    }
    return csc ? 'C' : csr ? 'R' : 'N';
}

typedef struct {
    int64_t major, minor, pos;
} orc_sort_key;

static int cmp_sort_key(const void *a, const void *b) {
    const orc_sort_key *x = (const orc_sort_key *)a, *y = (const orc_sort_key *)b;
    if (x->major != y->major) return x->major < y->major ? -1 : 1;
    if (x->minor != y->minor) return x->minor < y->minor ? -1 : 1;
    return x->pos < y->pos ? -1 : x->pos > y->pos;  /* equal keys keep their order */
}

/*
 * coo_arrays_apply_sort (sparse_data/base.hh:169-220): sort (vals, rows, cols) by (row, col)
 * for 'R' or (col, row) for 'C'; no-op for 'N' or when already in that order.  Equal keys keep
 * their relative order (the reference's std::sort leaves it unspecified).
 */
int orc_coo_apply_sort(int sort, int dtype, int itype, int64_t nnz, void *vals, void *rows,
                       void *cols) {
    if (sort == 'N' || orc_coo_determine_sort(itype, nnz, rows, cols) == sort) return 0;
    orc_sort_key *k = (orc_sort_key *)malloc(sizeof(orc_sort_key) * (size_t)(nnz > 0 ? nnz : 1));
    size_t vsz = dtype == ORC_F32 ? 4 : 8, isz = itype == ORC_I32 ? 4 : 8;
    char *tv = (char *)malloc(vsz * (size_t)(nnz > 0 ? nnz : 1));
    char *tr = (char *)malloc(isz * (size_t)(nnz > 0 ? nnz : 1));
    char *tc = (char *)malloc(isz * (size_t)(nnz > 0 ? nnz : 1));
    if (!k || !tv || !tr || !tc) { free(k); free(tv); free(tr); free(tc); return 2; }
    for (int64_t e = 0; e < nnz; ++e) {
        int64_t r = get_idx(itype, rows, e), c = get_idx(itype, cols, e);
        k[e].major = sort == 'R' ? r : c;
        k[e].minor = sort == 'R' ? c : r;
        k[e].pos = e;
    }
    qsort(k, (size_t)nnz, sizeof(orc_sort_key), cmp_sort_key);
    for (int64_t e = 0; e < nnz; ++e) {
        memcpy(tv + vsz * e, (char *)vals + vsz * k[e].pos, vsz);
        memcpy(tr + isz * e, (char *)rows + isz * k[e].pos, isz);
        memcpy(tc + isz * e, (char *)cols + isz * k[e].pos, isz);
    }
    memcpy(vals, tv, vsz * (size_t)nnz);
    memcpy(rows, tr, isz * (size_t)nnz);
    memcpy(cols, tc, isz * (size_t)nnz);
    free(k); free(tv); free(tr); free(tc);
    return 0;
}

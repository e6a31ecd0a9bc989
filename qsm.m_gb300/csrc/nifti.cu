// NIfTI-1 reading and writing as QSM.m does it: src/io/loadNii.m and saveNii.m
// over the NIfTI toolbox in third_party/NIfTI (load_nii.m, load_nii_hdr.m,
// load_nii_img.m, xform_nii.m, make_nii.m, save_nii.m, save_nii_hdr.m).
//
// The header logic runs on the host: parsing (either byte order), the
// scaling decision and the reorientation that load_nii applies from the sform
// or qform (xform_nii.m change_hdr / get_orient: a generalized permutation
// matrix after small entries are cleared, else an error), and the 352-byte
// header that saveNii writes.  The voxels go through one device pass: the
// stored bytes (host or device) are byte-swapped, scaled, converted, flipped
// and permuted into the loaded image in MATLAB order, so a volume read from
// disk lands in HBM ready for the solvers.  File access and gzip stay with the
// caller (the Python layer), as the MATLAB code leaves them to gunzip/fopen.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>

#include "common.cuh"

namespace qsm {
namespace {

// bytes per stored element and whether the datatype is one this path decodes
int elem_bytes(int dt)
{
    switch (dt) {
    case 2: case 256: return 1;                   // uint8, int8
    case 4: case 512: return 2;                   // int16, uint16
    case 8: case 16: case 768: return 4;          // int32, float32, uint32
    case 64: case 1024: case 1280: return 8;      // float64, int64, uint64
    default: return 0;                            // 1 (bit), 32/1792 (complex), 128/511 (RGB)
    }
}

// bitpix load_nii_img.m:read_image assigns per datatype (0: unsupported)
int bitpix_of(int dt)
{
    switch (dt) {
    case 1: return 1;
    case 2: case 256: return 8;
    case 4: case 512: return 16;
    case 8: case 16: case 768: return 32;
    case 32: case 64: case 1024: case 1280: return 64;
    case 128: return 24;
    case 511: return 96;
    case 1792: return 128;
    default: return 0;
    }
}

struct Reader {
    const uint8_t *b;
    bool swap;
    template <typename T> T get(size_t off) const
    {
        uint8_t t[sizeof(T)];
        for (size_t i = 0; i < sizeof(T); ++i) t[i] = b[off + (swap ? sizeof(T) - 1 - i : i)];
        T v;
        memcpy(&v, t, sizeof(T));
        return v;
    }
    void str(size_t off, size_t n, char *out) const  // deblank(fread(n, 'uchar=>char'))
    {
        memcpy(out, b + off, n);
        out[n] = 0;
        long e = (long)n - 1;
        while (e >= 0 && (out[e] == 0 || out[e] == ' ' || out[e] == '\t' || out[e] == '\n' || out[e] == '\r' ||
                          out[e] == '\v' || out[e] == '\f'))
            out[e--] = 0;
    }
};

qsm_status fail(qsm_nifti_hdr *h, qsm_status st, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(h->error, sizeof h->error, fmt, ap);
    va_end(ap);
    return st;
}

// R has exactly one non-zero per row and column, in the sense of xform_nii.m:
// det(R) != 0 and R(find(R)) == sum(R)' (one non-zero per column, column order)
bool gen_perm(const double R[3][3])
{
    const double det = R[0][0] * (R[1][1] * R[2][2] - R[1][2] * R[2][1]) -
                       R[0][1] * (R[1][0] * R[2][2] - R[1][2] * R[2][0]) +
                       R[0][2] * (R[1][0] * R[2][1] - R[1][1] * R[2][0]);
    if (det == 0.0) return false;
    for (int c = 0; c < 3; ++c) {
        int nz = 0;
        for (int r = 0; r < 3; ++r) nz += R[r][c] != 0.0;
        if (nz != 1) return false;
    }
    return true;
}

// clear entries below tolerance x the smallest of the three largest |R|
void clear_small(double R[3][3], double tol)
{
    double a[9];
    for (int i = 0; i < 9; ++i) a[i] = fabs(R[i % 3][i / 3]);
    std::sort(a, a + 9);
    const double lim = tol * std::min(std::min(a[6], a[7]), a[8]);
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c)
            if (fabs(R[r][c]) < lim) R[r][c] = 0.0;
}

qsm_status launch_status(qsm_ctx *ctx)
{
    QSM_CUDA(cudaGetLastError());
    return QSM_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
// device pass: stored bytes -> loaded image
// ---------------------------------------------------------------------------

struct Orient {
    int64_t m[3];    // stored spatial sizes
    int64_t n[3];    // loaded spatial sizes
    int perm[3];     // loaded axis j = stored axis perm[j]
    int flip[3];     // loaded axis j runs backwards
    int64_t total;   // elements
    int64_t rows;    // loaded rows: n[1] * n[2] * (extra dimensions)
    int swap;
};

// Rows of the loaded image, (64 x 4)-thread blocks: threadIdx.y picks a row,
// threadIdx.x strides along it.  The stored index of loaded (o0, o1, o2, t)
// is base(o1, o2, t) + step * o0 (step < 0 when loaded x runs backwards).
struct RowMap {
    int64_t base, step;
};

__device__ __forceinline__ RowMap row_map(const Orient &o, int64_t r)
{
    const int64_t o1 = r % o.n[1], r2 = r / o.n[1];
    const int64_t o2 = r2 % o.n[2], t = r2 / o.n[2];
    const int64_t st[3] = {1, o.m[0], o.m[0] * o.m[1]};
    const int64_t oj[3] = {0, o1, o2};
    int64_t base = t * o.m[0] * o.m[1] * o.m[2];
#pragma unroll
    for (int j = 1; j < 3; ++j) {
        const int a = o.perm[j];
        base += st[a] * (o.flip[j] ? o.m[a] - 1 - oj[j] : oj[j]);
    }
    const int a0 = o.perm[0];
    RowMap rm;
    rm.base = base + (o.flip[0] ? st[a0] * (o.m[a0] - 1) : 0);
    rm.step = o.flip[0] ? -st[a0] : st[a0];
    return rm;
}

template <int B> struct Word;
template <> struct Word<1> { using T = uint8_t; __device__ static T bswap(T x) { return x; } };
template <> struct Word<2> {
    using T = uint16_t;
    __device__ static T bswap(T x) { return (T)((x >> 8) | (x << 8)); }
};
template <> struct Word<4> {
    using T = uint32_t;
    __device__ static T bswap(T x) { return __byte_perm(x, 0u, 0x0123); }
};
template <> struct Word<8> {
    using T = unsigned long long;
    __device__ static T bswap(T x)
    {
        const uint32_t lo = (uint32_t)x, hi = (uint32_t)(x >> 32);
        return ((T)__byte_perm(lo, 0u, 0x0123) << 32) | (T)__byte_perm(hi, 0u, 0x0123);
    }
};

template <typename S>
__device__ __forceinline__ S load_elem(const S *__restrict__ p, int64_t i, int swap)
{
    using W = Word<sizeof(S)>;
    typename W::T w = __ldg((const typename W::T *)p + i);
    if (swap) w = W::bswap(w);
    S v;
    memcpy(&v, &w, sizeof(S));
    return v;
}

// the loaded class unchanged: a reoriented, byte-order-corrected copy
template <int B>
__global__ void __launch_bounds__(256) copy_k(typename Word<B>::T *__restrict__ out,
                                              const typename Word<B>::T *__restrict__ in, Orient o)
{
    using W = Word<B>;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.y + threadIdx.y; r < o.rows; r += (int64_t)gridDim.x * blockDim.y) {
        const RowMap rm = row_map(o, r);
        typename W::T *dst = out + r * o.n[0];
        for (int64_t x = threadIdx.x; x < o.n[0]; x += blockDim.x) {
            typename W::T w = __ldg(in + rm.base + rm.step * x);
            dst[x] = o.swap ? W::bswap(w) : w;
        }
    }
}

// converted (and, when load_nii scales, scl_slope * double(x) + scl_inter,
// rounded to single unless the stored class is double)
template <typename S, typename O>
__global__ void __launch_bounds__(256) convert_k(O *__restrict__ out, const S *__restrict__ in, Orient o, int scaled,
                                                 double slope, double inter, int to_single)
{
    for (int64_t r = (int64_t)blockIdx.x * blockDim.y + threadIdx.y; r < o.rows; r += (int64_t)gridDim.x * blockDim.y) {
        const RowMap rm = row_map(o, r);
        O *dst = out + r * o.n[0];
        for (int64_t x = threadIdx.x; x < o.n[0]; x += blockDim.x) {
            const S v = load_elem<S>(in, rm.base + rm.step * x, o.swap);
            if (scaled) {
                const double w = slope * (double)v + inter;
                dst[x] = to_single ? (O)(float)w : (O)w;
            } else {
                dst[x] = (O)v;
            }
        }
    }
}

// scaled 8- and 16-bit images: every stored value's result, computed once as
// load_nii computes it (FP64 scl_slope * x + scl_inter, then single), indexed
// by the stored bits; FP64 per voxel would bind the pass to the FP64 pipe
template <typename S, typename O>
__global__ void scale_table_k(O *__restrict__ tab, double slope, double inter, int to_single)
{
    using W = typename Word<sizeof(S)>::T;
    const unsigned n = 1u << (8 * sizeof(S));
    for (unsigned u = blockIdx.x * blockDim.x + threadIdx.x; u < n; u += gridDim.x * blockDim.x) {
        const W w = (W)u;
        S v;
        memcpy(&v, &w, sizeof(S));
        const double r = slope * (double)v + inter;
        tab[u] = to_single ? (O)(float)r : (O)r;
    }
}

template <typename S, typename O>
__global__ void __launch_bounds__(256) lookup_k(O *__restrict__ out, const S *__restrict__ in,
                                                const O *__restrict__ tab, Orient o)
{
    using W = Word<sizeof(S)>;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.y + threadIdx.y; r < o.rows; r += (int64_t)gridDim.x * blockDim.y) {
        const RowMap rm = row_map(o, r);
        O *dst = out + r * o.n[0];
        for (int64_t x = threadIdx.x; x < o.n[0]; x += blockDim.x) {
            typename W::T w = __ldg((const typename W::T *)in + rm.base + rm.step * x);
            if (o.swap) w = W::bswap(w);
            dst[x] = __ldg(tab + w);
        }
    }
}

// max and min over the non-NaN elements of an image (for glmax / glmin)
// order-preserving 64-bit key of a double
__device__ __forceinline__ unsigned long long order_key(double d)
{
    const unsigned long long u = (unsigned long long)__double_as_longlong(d);
    return (u >> 63) ? ~u : (u | 0x8000000000000000ull);
}

template <typename T> struct Cmp {  // integers and float compare in their own type
    __device__ static bool nan(T v) { return v != v; }
    __device__ static bool less(T a, T b) { return a < b; }
};
template <> struct Cmp<double> {     // doubles by their bits (no FP64 instruction per element)
    __device__ static bool nan(double v)
    {
        const unsigned long long u = (unsigned long long)__double_as_longlong(v);
        return (u & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
    }
    __device__ static bool less(double a, double b) { return order_key(a) < order_key(b); }
};

template <typename T>
__global__ void minmax_k(const T *__restrict__ a, int64_t n, unsigned long long *mx, unsigned long long *mn,
                         int *any)
{
    T hi = 0, lo = 0;
    int seen = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const T v = a[i];
        if (Cmp<T>::nan(v)) continue;
        if (!seen || Cmp<T>::less(hi, v)) hi = v;
        if (!seen || Cmp<T>::less(v, lo)) lo = v;
        seen = 1;
    }
    // block reduction of the keys (warp shuffles, then warp 0), one atomic per block
    unsigned long long kh = seen ? order_key((double)hi) : 0ull, kl = seen ? order_key((double)lo) : ~0ull;
#pragma unroll
    for (int s = 16; s > 0; s >>= 1) {
        kh = max(kh, __shfl_xor_sync(0xffffffffu, kh, s));
        kl = min(kl, __shfl_xor_sync(0xffffffffu, kl, s));
    }
    __shared__ unsigned long long sh[2][32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
    if (lane == 0) {
        sh[0][wid] = kh;
        sh[1][wid] = kl;
    }
    __syncthreads();
    if (wid == 0) {
        kh = lane < nw ? sh[0][lane] : 0ull;
        kl = lane < nw ? sh[1][lane] : ~0ull;
#pragma unroll
        for (int s = 16; s > 0; s >>= 1) {
            kh = max(kh, __shfl_xor_sync(0xffffffffu, kh, s));
            kl = min(kl, __shfl_xor_sync(0xffffffffu, kl, s));
        }
        if (lane == 0 && kl != ~0ull) {  // a non-NaN element was seen in this block
            atomicMax(mx, kh);
            atomicMin(mn, kl);
            atomicOr(any, 1);
        }
    }
}

}  // namespace qsm

using namespace qsm;

extern "C" {

qsm_status qsm_nifti_parse(const void *bytes, size_t nbytes, double tolerance, char preferred_form,
                           qsm_nifti_hdr *h)
{
    if (!h) return QSM_ERR_ARG;
    memset(h, 0, sizeof *h);
    if (!bytes) return fail(h, QSM_ERR_ARG, "no header bytes");
    if (nbytes < 348) return fail(h, QSM_ERR_ARG, "a NIfTI-1 header has 348 bytes, got %zu", nbytes);
    // load_nii_hdr.m: little-endian first, then big-endian; sizeof_hdr must read 348
    Reader r{(const uint8_t *)bytes, false};
    if (r.get<int32_t>(0) != 348) {
        r.swap = true;
        if (r.get<int32_t>(0) != 348) return fail(h, QSM_ERR_ARG, "file is corrupted (sizeof_hdr is not 348)");
    }
    h->big_endian = r.swap ? 1 : 0;
    r.str(4, 10, h->data_type);
    r.str(14, 18, h->db_name);
    int16_t dim[8];
    for (int i = 0; i < 8; ++i) dim[i] = r.get<int16_t>(40 + 2 * i);
    h->stored_datatype = r.get<int16_t>(70);
    double pix[8];
    for (int i = 0; i < 8; ++i) pix[i] = (double)r.get<float>(76 + 4 * i);
    h->vox_offset_stored = (double)r.get<float>(108);
    h->scl_slope = (double)r.get<float>(112);
    h->scl_inter = (double)r.get<float>(116);
    int xyzt = r.get<uint8_t>(123);
    r.str(148, 80, h->descrip);
    r.str(228, 24, h->aux_file);
    h->qform_code = r.get<int16_t>(252);
    h->sform_code = r.get<int16_t>(254);
    for (int i = 0; i < 3; ++i) h->quatern[i] = (double)r.get<float>(256 + 4 * i);
    for (int i = 0; i < 3; ++i) h->qoffset[i] = (double)r.get<float>(268 + 4 * i);
    for (int i = 0; i < 12; ++i) h->srow[i] = (double)r.get<float>(280 + 4 * i);
    r.str(328, 16, h->intent_name);
    r.str(344, 4, h->magic);
    for (int i = 0; i < 5; ++i) h->originator[i] = (double)r.get<int16_t>(253 + 2 * i);
    const bool nifti = !strcmp(h->magic, "n+1") || !strcmp(h->magic, "ni1");
    if (!nifti) h->qform_code = h->sform_code = 0;
    h->filetype = !strcmp(h->magic, "n+1") ? 2 : !strcmp(h->magic, "ni1") ? 1 : 0;

    // load_nii_img.m:read_image
    h->bitpix = bitpix_of(h->stored_datatype);
    if (!h->bitpix) return fail(h, QSM_ERR_DTYPE, "datatype %d is not supported", h->stored_datatype);
    for (int i = 0; i < 8; ++i) h->stored_dim[i] = dim[i] < 1 ? 1 : dim[i];
    {
        // seven int16 sizes can multiply past any buffer: refuse images over 2^40 elements
        double n = 1.0;
        for (int i = 1; i < 8; ++i) n *= (double)h->stored_dim[i];
        if (n > 1099511627776.0) return fail(h, QSM_ERR_DIMS, "image of %.3g elements is too large", n);
    }
    h->vox_offset = h->filetype == 2 ? (int64_t)h->vox_offset_stored : 0;
    h->datatype = h->stored_datatype;

    // xform_nii.m: scaling of real integer / float images
    const int sdt = h->stored_datatype;
    const bool scalable = sdt == 2 || sdt == 4 || sdt == 8 || sdt == 16 || sdt == 64 || sdt == 256 || sdt == 512 ||
                          sdt == 768;
    if (h->scl_slope != 0.0 && scalable && (h->scl_slope != 1.0 || h->scl_inter != 0.0)) {
        h->scaled = 1;
        h->datatype = sdt == 64 ? 64 : 16;
    } else if (h->scl_slope != 0.0 && (sdt == 32 || sdt == 1792)) {
        h->scaled = 1;
    }
    for (int i = 0; i < 8; ++i) {
        h->dim[i] = h->stored_dim[i];
        h->pixdim[i] = pix[i];
    }
    h->xyzt_units = xyzt;
    for (int j = 0; j < 3; ++j) h->perm[j] = j;
    if (h->filetype == 0) return QSM_OK;  // Analyze 7.5: no sform/qform (an SPM .mat is not read)

    // change_hdr
    if (tolerance <= 0.0) tolerance = 2.220446049250313e-16;
    char use = 0;
    if (preferred_form == 'S') {
        if (h->sform_code == 0) return fail(h, QSM_ERR_ARG, "User requires sform, sform not set in header");
        use = 's';
    } else if (preferred_form == 'Q') {
        if (h->qform_code == 0) return fail(h, QSM_ERR_ARG, "User requires qform, qform not set in header");
        use = 'q';
    } else if (preferred_form == 'q') {
        use = h->qform_code > 0 ? 'q' : h->sform_code > 0 ? 's' : 0;
    } else {
        use = h->sform_code > 0 ? 's' : h->qform_code > 0 ? 'q' : 0;
    }
    const char *shear = "Non-orthogonal rotation or shearing found inside the affine matrix in this NIfTI file";
    double R[3][3], T[3];
    if (use == 's') {
        for (int i = 0; i < 3; ++i) {
            for (int c = 0; c < 3; ++c) R[i][c] = h->srow[4 * i + c];
            T[i] = h->srow[4 * i + 3];
        }
        if (!gen_perm(R)) {
            clear_small(R, tolerance);
            if (!gen_perm(R)) return fail(h, QSM_ERR_ARG, "%s", shear);
        }
    } else if (use == 'q') {
        const double b = h->quatern[0], c = h->quatern[1], d = h->quatern[2];
        double a;
        if (1.0 - (b * b + c * c + d * d) < 0.0) {
            if (fabs(1.0 - (b * b + c * c + d * d)) < 1e-5) a = 0.0;
            else return fail(h, QSM_ERR_ARG, "Incorrect quaternion values in this NIFTI data.");
        } else {
            a = sqrt(1.0 - (b * b + c * c + d * d));
        }
        double qfac = pix[0];
        if (qfac == 0.0) qfac = 1.0;
        const double sc[3] = {pix[1], pix[2], qfac * pix[3]};
        R[0][0] = a * a + b * b - c * c - d * d; R[0][1] = 2 * b * c - 2 * a * d;  R[0][2] = 2 * b * d + 2 * a * c;
        R[1][0] = 2 * b * c + 2 * a * d;  R[1][1] = a * a + c * c - b * b - d * d; R[1][2] = 2 * c * d - 2 * a * b;
        R[2][0] = 2 * b * d - 2 * a * c;  R[2][1] = 2 * c * d + 2 * a * b;  R[2][2] = a * a + d * d - c * c - b * b;
        for (int i = 0; i < 3; ++i) T[i] = h->qoffset[i];
        if (!gen_perm(R)) {
            clear_small(R, tolerance);
            for (int i = 0; i < 3; ++i)
                for (int k = 0; k < 3; ++k) R[i][k] *= sc[k];
            if (!gen_perm(R)) return fail(h, QSM_ERR_ARG, "%s", shear);
        } else {
            for (int i = 0; i < 3; ++i)
                for (int k = 0; k < 3; ++k) R[i][k] *= sc[k];
        }
    }
    int orient[3] = {1, 2, 3};
    if (use) {
        // voxel_size = abs(sum(R, 1)); inv(R) of a generalized permutation matrix;
        // originator = inv(R) * -T + 1; orient from the rows of inv(R) (get_orient)
        for (int c = 0; c < 3; ++c) h->pixdim[1 + c] = fabs(R[0][c] + R[1][c] + R[2][c]);
        for (int c = 0; c < 3; ++c) {
            int rr = 0;
            for (int i = 0; i < 3; ++i)
                if (R[i][c] != 0.0) rr = i;
            const double inv = 1.0 / R[rr][c];  // inv(R)(c, rr)
            h->originator[c] = inv * -T[rr] + 1.0;
            orient[c] = inv > 0.0 ? rr + 1 : rr + 4;
        }
        h->qform_code = h->sform_code = 0;
    }
    // get_units: metres and micrometres become millimetres
    const int su = xyzt & 7;
    const double space_unit = su == 1 ? 1e3 : su == 3 ? 1e-3 : 1.0;
    if (space_unit != 1.0) {
        for (int c = 1; c <= 3; ++c) h->pixdim[c] *= space_unit;
        h->xyzt_units = (xyzt & ~7) | 2;
    }
    for (int i = 0; i < 8; ++i) h->pixdim[i] = fabs(h->pixdim[i]);

    // xform_nii.m: flip stored axes that run backwards, then sort axes into x, y, z
    if (!(orient[0] == 1 && orient[1] == 2 && orient[2] == 3)) {
        int rot0[3], flip0[3];
        for (int i = 0; i < 3; ++i) {
            rot0[i] = (orient[i] + 2) % 3 + 1;
            flip0[i] = orient[i] - rot0[i] != 0;
        }
        int perm[3] = {0, 1, 2};
        std::stable_sort(perm, perm + 3, [&](int x, int y) { return rot0[x] < rot0[y]; });
        const int64_t old_dim[3] = {h->stored_dim[1], h->stored_dim[2], h->stored_dim[3]};
        const double old_pix[3] = {h->pixdim[1], h->pixdim[2], h->pixdim[3]};
        const double old_org[3] = {h->originator[0], h->originator[1], h->originator[2]};
        for (int j = 0; j < 3; ++j) {
            h->perm[j] = perm[j];
            h->flip[j] = flip0[perm[j]];
            h->dim[1 + j] = old_dim[perm[j]];
            h->pixdim[1 + j] = old_pix[perm[j]];
            double t = old_org[perm[j]];
            if (h->flip[j] && t != 0.0) t = (double)h->dim[1 + j] - t + 1.0;
            h->originator[j] = t;
        }
        h->reoriented = 1;
    }
    return QSM_OK;
}

size_t qsm_nifti_payload_bytes(const qsm_nifti_hdr *h)
{
    if (!h) return 0;
    size_t n = 1;
    for (int i = 1; i < 8; ++i) n *= (size_t)h->stored_dim[i];
    return n * (size_t)h->bitpix / 8;
}

qsm_status qsm_nifti_decode(qsm_ctx *ctx, const qsm_nifti_hdr *h, const void *payload, int32_t out_datatype,
                            void *img)
{
    Range nvtx_range("nifti_decode");
    if (!ctx || !h || !payload || !img) return QSM_ERR_ARG;
    const int sdt = h->stored_datatype, eb = elem_bytes(sdt);
    if (!eb) return set_error(ctx, "datatype %d (bit, complex or RGB) is not decoded", sdt), QSM_ERR_DTYPE;
    if (out_datatype == 0) out_datatype = h->datatype;
    if (out_datatype != h->datatype && out_datatype != 16 && out_datatype != 64)
        return set_error(ctx, "out_datatype must be 0, 16, 64 or the loaded datatype"), QSM_ERR_DTYPE;
    cudaSetDevice(ctx->device);
    Orient o;
    o.total = 1;
    for (int i = 1; i < 8; ++i) o.total *= h->stored_dim[i];
    for (int a = 0; a < 3; ++a) {
        o.m[a] = h->stored_dim[1 + a];
        o.n[a] = h->dim[1 + a];
        o.perm[a] = h->perm[a];
        o.flip[a] = h->flip[a];
    }
    o.swap = h->big_endian;
    const size_t in_bytes = (size_t)o.total * eb;
    const int ob = out_datatype == 64 ? 8 : out_datatype == 16 ? 4 : eb;
    Staged si, so;
    QSM_TRY(stage_in(ctx, si, payload, in_bytes, true));
    qsm_status st = stage_in(ctx, so, img, (size_t)o.total * ob, false);
    if (st != QSM_OK) {
        stage_out(ctx, si, false);
        return st;
    }
    // element loads and stores are whole words: device buffers given by the caller
    // must be aligned to their element size (staged host buffers always are)
    if (((uintptr_t)si.dev % eb) || ((uintptr_t)so.dev % ob)) {
        stage_out(ctx, si, false);
        stage_out(ctx, so, false);
        set_error(ctx, "payload and image must be aligned to their element sizes (%d, %d bytes)", eb, ob);
        return QSM_ERR_ARG;
    }
    o.rows = o.total / o.n[0];
    const dim3 blk(64, 4);
    const unsigned g = (unsigned)std::min<int64_t>((o.rows + 3) / 4, 152 * 16);
    const void *in = si.dev;
    const bool to_single = h->datatype == 16;
    if (!h->scaled && out_datatype == h->datatype) {
        switch (eb) {
        case 1: copy_k<1><<<g, blk, 0, ctx->stream>>>((uint8_t *)so.dev, (const uint8_t *)in, o); break;
        case 2: copy_k<2><<<g, blk, 0, ctx->stream>>>((uint16_t *)so.dev, (const uint16_t *)in, o); break;
        case 4: copy_k<4><<<g, blk, 0, ctx->stream>>>((uint32_t *)so.dev, (const uint32_t *)in, o); break;
        default:
            copy_k<8><<<g, blk, 0, ctx->stream>>>((unsigned long long *)so.dev, (const unsigned long long *)in, o);
            break;
        }
    } else if (h->scaled && eb <= 2) {
        const size_t nt = (size_t)1 << (8 * eb);
        void *tab = nullptr;
        st = dalloc(ctx, &tab, nt * ob);
        if (st != QSM_OK) {
            stage_out(ctx, si, false);
            stage_out(ctx, so, false);
            return st;
        }
#define QSM_LOOKUP(S, O)                                                                                         \
    scale_table_k<S, O><<<(unsigned)((nt + 255) / 256), 256, 0, ctx->stream>>>((O *)tab, h->scl_slope,          \
                                                                             h->scl_inter, to_single);        \
    lookup_k<S, O><<<g, blk, 0, ctx->stream>>>((O *)so.dev, (const S *)in, (const O *)tab, o);
#define QSM_LOOKUP2(S)                                                                                           \
    if (out_datatype == 64) { QSM_LOOKUP(S, double) } else { QSM_LOOKUP(S, float) }
        switch (sdt) {
        case 2: QSM_LOOKUP2(uint8_t) break;
        case 256: QSM_LOOKUP2(int8_t) break;
        case 4: QSM_LOOKUP2(int16_t) break;
        default: QSM_LOOKUP2(uint16_t) break;
        }
#undef QSM_LOOKUP2
#undef QSM_LOOKUP
        dfree(ctx, tab);
    } else {
#define QSM_CONVERT(S)                                                                                           \
    if (out_datatype == 64)                                                                                      \
        convert_k<S, double><<<g, blk, 0, ctx->stream>>>((double *)so.dev, (const S *)in, o, h->scaled,          \
                                                         h->scl_slope, h->scl_inter, to_single);                 \
    else                                                                                                         \
        convert_k<S, float><<<g, blk, 0, ctx->stream>>>((float *)so.dev, (const S *)in, o, h->scaled,            \
                                                        h->scl_slope, h->scl_inter, to_single);
        switch (sdt) {
        case 2: QSM_CONVERT(uint8_t) break;
        case 256: QSM_CONVERT(int8_t) break;
        case 4: QSM_CONVERT(int16_t) break;
        case 512: QSM_CONVERT(uint16_t) break;
        case 8: QSM_CONVERT(int32_t) break;
        case 768: QSM_CONVERT(uint32_t) break;
        case 16: QSM_CONVERT(float) break;
        case 64: QSM_CONVERT(double) break;
        case 1024: QSM_CONVERT(int64_t) break;
        default: QSM_CONVERT(uint64_t) break;
        }
#undef QSM_CONVERT
    }
    st = launch_status(ctx);
    stage_out(ctx, si, false);
    qsm_status st2 = stage_out(ctx, so, st == QSM_OK);
    if (st == QSM_OK) st = st2;
    if (st == QSM_OK) {
        cudaError_t e = cudaStreamSynchronize(ctx->stream);
        if (e != cudaSuccess) return set_error(ctx, "%s", cudaGetErrorString(e)), QSM_ERR_CUDA;
    }
    return st;
}

qsm_status qsm_nifti_make_header(qsm_ctx *ctx, int32_t datatype, int32_t ndims, const int64_t *size,
                                 const double vsz[3], int32_t filetype, const void *img, uint8_t *hdr_out)
{
    if (!ctx || !size || !vsz || !hdr_out || ndims < 1 || (filetype != 1 && filetype != 2)) return QSM_ERR_ARG;
    if (ndims > 7) return set_error(ctx, "NIfTI only allows a maximum of 7 Dimension matrix."), QSM_ERR_DIMS;
    const int eb = elem_bytes(datatype);
    if (!eb || datatype == 1024 || datatype == 1280)
        return set_error(ctx, "Datatype is not supported by make_nii."), QSM_ERR_DTYPE;
    // dims = [ndims(img) size(img) 1 ...](1:8); MATLAB's size drops trailing singletons
    int nd = ndims;
    while (nd > 2 && size[nd - 1] == 1) --nd;
    if (nd < 2) nd = 2;
    int64_t n = 1;
    for (int i = 0; i < ndims; ++i) {
        if (size[i] < 0) return QSM_ERR_DIMS;
        n *= size[i];
    }
    // glmax / glmin = round(double(max / min of the image)) (make_nii.m, save_nii.m)
    double gmax = 0.0, gmin = 0.0;
    bool have = false;
    if (n > 0) {
        if (!img) return QSM_ERR_ARG;
        cudaSetDevice(ctx->device);
        Staged si;
        QSM_TRY(stage_in(ctx, si, img, (size_t)n * eb, true));
        void *scratch = nullptr;
        qsm_status st = dalloc(ctx, &scratch, 64);
        if (st != QSM_OK) {
            stage_out(ctx, si, false);
            return st;
        }
        unsigned long long *mx = (unsigned long long *)scratch, *mn = mx + 1;
        int *any = (int *)(mx + 2);
        const unsigned long long init[3] = {0ull, ~0ull, 0ull};
        cudaMemcpyAsync(scratch, init, sizeof init, cudaMemcpyHostToDevice, ctx->stream);
        const unsigned g = (unsigned)std::min<int64_t>((n + 255) / 256, 152 * 8);
#define QSM_MM(T) minmax_k<T><<<g, 256, 0, ctx->stream>>>((const T *)si.dev, n, mx, mn, any)
        switch (datatype) {
        case 2: QSM_MM(uint8_t); break;
        case 256: QSM_MM(int8_t); break;
        case 4: QSM_MM(int16_t); break;
        case 512: QSM_MM(uint16_t); break;
        case 8: QSM_MM(int32_t); break;
        case 768: QSM_MM(uint32_t); break;
        case 16: QSM_MM(float); break;
        default: QSM_MM(double); break;
        }
#undef QSM_MM
        unsigned long long res[3];
        st = launch_status(ctx);
        if (st == QSM_OK) {
            cudaError_t e = cudaMemcpyAsync(res, scratch, sizeof res, cudaMemcpyDeviceToHost, ctx->stream);
            if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
            if (e != cudaSuccess) st = (set_error(ctx, "%s", cudaGetErrorString(e)), QSM_ERR_CUDA);
        }
        dfree(ctx, scratch);
        stage_out(ctx, si, false);
        QSM_TRY(st);
        if ((int)res[2]) {
            auto dec = [](unsigned long long k) {
                const unsigned long long u = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
                double d;
                memcpy(&d, &u, 8);
                return d;
            };
            gmax = dec(res[0]);
            gmin = dec(res[1]);
            have = true;
        }
    }
    // MATLAB round (half away from zero), then fwrite 'int32' (saturating; NaN -> 0)
    auto to_i32 = [](double v) -> int32_t {
        v = v < 0 ? -floor(-v + 0.5) : floor(v + 0.5);
        if (v != v) return 0;
        if (v > 2147483647.0) return 2147483647;
        if (v < -2147483648.0) return (int32_t)-2147483647 - 1;
        return (int32_t)v;
    };
    const int32_t glmax = have ? to_i32(gmax) : 0, glmin = have ? to_i32(gmin) : 0;
    auto i16 = [](int64_t v) -> int16_t { return (int16_t)std::min<int64_t>(std::max<int64_t>(v, -32768), 32767); };

    uint8_t *b = hdr_out;
    memset(b, 0, filetype == 2 ? 352 : 348);
    auto put = [&](size_t off, const void *v, size_t k) { memcpy(b + off, v, k); };
    auto p32 = [&](size_t off, int32_t v) { put(off, &v, 4); };
    auto p16 = [&](size_t off, int16_t v) { put(off, &v, 2); };
    auto pf = [&](size_t off, double v) { const float f = (float)v; put(off, &f, 4); };
    p32(0, 348);            // sizeof_hdr
    b[38] = 'r';            // regular
    int16_t dim[8] = {(int16_t)nd, 1, 1, 1, 1, 1, 1, 1};
    for (int i = 0; i < nd && i < 7; ++i) dim[1 + i] = i16(i < ndims ? size[i] : 1);
    for (int i = 0; i < 8; ++i) p16(40 + 2 * i, dim[i]);
    p16(70, (int16_t)datatype);
    p16(72, (int16_t)bitpix_of(datatype));
    const double pixdim[8] = {0.0, vsz[0], vsz[1], vsz[2], 1.0, 1.0, 1.0, 1.0};
    for (int i = 0; i < 8; ++i) pf(76 + 4 * i, pixdim[i]);
    pf(108, filetype == 2 ? 352.0 : 0.0);  // vox_offset
    p32(140, glmax);
    p32(144, glmin);
    memcpy(b + 228, "none", 4);  // aux_file
    // save_nii_hdr.m: neither qform nor sform -> sform_code 1 from pixdim and originator 0
    p16(254, 1);
    const double srow[12] = {pixdim[1], 0.0, 0.0, (1.0 - 0.0) * pixdim[1], 0.0, pixdim[2], 0.0, (1.0 - 0.0) * pixdim[2],
                             0.0, 0.0, pixdim[3], (1.0 - 0.0) * pixdim[3]};
    for (int i = 0; i < 12; ++i) pf(280 + 4 * i, srow[i]);
    memcpy(b + 344, filetype == 2 ? "n+1" : "ni1", 4);  // magic (with its terminating zero)
    return QSM_OK;
}

}  // extern "C"

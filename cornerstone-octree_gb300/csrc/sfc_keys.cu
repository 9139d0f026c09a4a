// SFC key encoding and permutation gathers.
//
// Keys: one pass over x, y, z (SoA), 4 particles per thread with 16-byte vector loads where the arrays are aligned,
// sfc3D quantisation with unfused arithmetic (sfc/sfc.hpp:142-179), Hilbert keys through the state table in shared
// memory (one lookup per level) or Morton interleave, 16-byte stores.
// HBM-bound: 3*sizeof(T) + sizeof(K) bytes per particle (+ sizeof(K) when removeKey entries are respected).
#include "cs_common.cuh"
#include "sfc_keys.cuh"

#include <type_traits>

namespace csg
{

// the Hilbert state table (iHilbertByTable), staged into shared memory by the key kernels of the Hilbert curve
__device__ const HilbertTable kHilbertTable = makeHilbertTable();

template<int Kind>
__device__ __forceinline__ const uint16_t* stageHilbertTable(uint16_t* sH)
{
    if constexpr (Kind == CS_HILBERT)
    {
        for (int i = threadIdx.x; i < 384; i += blockDim.x)
            sH[i] = kHilbertTable.e[i];
        __syncthreads();
        return sH;
    }
    else { return nullptr; }
}

template<class T, class K, int Kind, bool RespectRemove>
__global__ void __launch_bounds__(256) sfcKeysKernel(const T* __restrict__ x, const T* __restrict__ y,
                                                     const T* __restrict__ z, K* __restrict__ keys, size_t n,
                                                     KeyParams<T, K> p)
{
    __shared__ uint16_t sH[384];
    const uint16_t* ht = stageHilbertTable<Kind>(sH);
    constexpr int V = 4;
    size_t stride   = size_t(gridDim.x) * blockDim.x;
    for (size_t base = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) * V; base < n; base += stride * V)
    {
        if (base + V <= n)
        {
            T xs[V], ys[V], zs[V];
#pragma unroll
            for (int v = 0; v < V; ++v)
            {
                xs[v] = __ldcs(x + base + v);
                ys[v] = __ldcs(y + base + v);
                zs[v] = __ldcs(z + base + v);
            }
            K out[V];
#pragma unroll
            for (int v = 0; v < V; ++v)
            {
                K k = sfc3D<T, K>(xs[v], ys[v], zs[v], p, Kind, ht);
                if constexpr (RespectRemove)
                {
                    K old = keys[base + v];
                    if (old == removeKey<K>()) k = old;
                }
                out[v] = k;
            }
#pragma unroll
            for (int v = 0; v < V; ++v)
                keys[base + v] = out[v];
        }
        else
        {
            for (size_t i = base; i < n; ++i)
            {
                K k = sfc3D<T, K>(x[i], y[i], z[i], p, Kind, ht);
                if constexpr (RespectRemove)
                {
                    if (keys[i] == removeKey<K>()) continue;
                }
                keys[i] = k;
            }
        }
    }
}

template<class T, class K>
int sfcKeys(cudaStream_t s, const T* x, const T* y, const T* z, K* keys, size_t n, const cs_box& box, int kind,
            bool respectRemove)
{
    if (n == 0) return CS_OK;
    if (!x || !y || !z || !keys)
    {
        setLastError("sfc keys: null pointer");
        return CS_ERR_INVALID;
    }
    auto bp        = makeBoxParams<T>(box);
    auto kp        = makeKeyParams<T, K>(bp);
    unsigned thr   = 256;
    size_t blocksN = (n + 4 * thr - 1) / (4 * thr);
    unsigned grid  = unsigned(blocksN < size_t(smCount()) * 16 ? blocksN : size_t(smCount()) * 16);
    if (kind == CS_HILBERT)
    {
        if (respectRemove) sfcKeysKernel<T, K, CS_HILBERT, true><<<grid, thr, 0, s>>>(x, y, z, keys, n, kp);
        else sfcKeysKernel<T, K, CS_HILBERT, false><<<grid, thr, 0, s>>>(x, y, z, keys, n, kp);
    }
    else
    {
        if (respectRemove) sfcKeysKernel<T, K, CS_MORTON, true><<<grid, thr, 0, s>>>(x, y, z, keys, n, kp);
        else sfcKeysKernel<T, K, CS_MORTON, false><<<grid, thr, 0, s>>>(x, y, z, keys, n, kp);
    }
    CSG_CHECK_LAUNCH();
    return CS_OK;
}

template int sfcKeys(cudaStream_t, const float*, const float*, const float*, uint32_t*, size_t, const cs_box&, int, bool);
template int sfcKeys(cudaStream_t, const double*, const double*, const double*, uint32_t*, size_t, const cs_box&, int,
                     bool);
template int sfcKeys(cudaStream_t, const float*, const float*, const float*, uint64_t*, size_t, const cs_box&, int, bool);
template int sfcKeys(cudaStream_t, const double*, const double*, const double*, uint64_t*, size_t, const cs_box&, int,
                     bool);

// keys of the pipeline: as sfcKeysKernel, and x, y, z, h written as one record per particle, so that the gather after
// the sort reads one sector per particle instead of four
template<class T, class K, int Kind>
__global__ void __launch_bounds__(256) sfcKeysPackKernel(const T* __restrict__ x, const T* __restrict__ y,
                                                         const T* __restrict__ z, const T* __restrict__ h,
                                                         K* __restrict__ keys, PackedT<T>* __restrict__ packed,
                                                         size_t n, KeyParams<T, K> p)
{
    __shared__ uint16_t sH[384];
    const uint16_t* ht = stageHilbertTable<Kind>(sH);
    constexpr int V = 4;
    size_t stride   = size_t(gridDim.x) * blockDim.x;
    for (size_t base = (size_t(blockIdx.x) * blockDim.x + threadIdx.x) * V; base < n; base += stride * V)
    {
        int m = int(n - base < V ? n - base : V);
        T xs[V], ys[V], zs[V], hs[V];
#pragma unroll
        for (int v = 0; v < V; ++v)
        {
            if (v < m)
            {
                xs[v] = __ldcs(x + base + v);
                ys[v] = __ldcs(y + base + v);
                zs[v] = __ldcs(z + base + v);
                hs[v] = __ldcs(h + base + v);
            }
        }
#pragma unroll
        for (int v = 0; v < V; ++v)
        {
            if (v < m)
            {
                keys[base + v]   = sfc3D<T, K>(xs[v], ys[v], zs[v], p, Kind, ht);
                PackedT<T> r;
                r.x              = xs[v];
                r.y              = ys[v];
                r.z              = zs[v];
                r.w              = hs[v];
                packed[base + v] = r;
            }
        }
    }
}

template<class T, class K>
int sfcKeysPacked(cudaStream_t s, const T* x, const T* y, const T* z, const T* h, K* keys, PackedT<T>* packed,
                  size_t n, const cs_box& box, int kind)
{
    if (n == 0) return CS_OK;
    auto bp        = makeBoxParams<T>(box);
    auto kp        = makeKeyParams<T, K>(bp);
    unsigned thr   = 256;
    size_t blocksN = (n + 4 * thr - 1) / (4 * thr);
    unsigned grid  = unsigned(blocksN < size_t(smCount()) * 16 ? blocksN : size_t(smCount()) * 16);
    if (kind == CS_HILBERT)
        sfcKeysPackKernel<T, K, CS_HILBERT><<<grid, thr, 0, s>>>(x, y, z, h, keys, packed, n, kp);
    else
        sfcKeysPackKernel<T, K, CS_MORTON><<<grid, thr, 0, s>>>(x, y, z, h, keys, packed, n, kp);
    CSG_CHECK_LAUNCH();
    return CS_OK;
}

template int sfcKeysPacked(cudaStream_t, const float*, const float*, const float*, const float*, uint32_t*, float4*,
                           size_t, const cs_box&, int);
template int sfcKeysPacked(cudaStream_t, const double*, const double*, const double*, const double*, uint32_t*,
                           double4_32a*, size_t, const cs_box&, int);
template int sfcKeysPacked(cudaStream_t, const float*, const float*, const float*, const float*, uint64_t*, float4*,
                           size_t, const cs_box&, int);
template int sfcKeysPacked(cudaStream_t, const double*, const double*, const double*, const double*, uint64_t*,
                           double4_32a*, size_t, const cs_box&, int);

template<class T, int Kind>
__global__ void __launch_bounds__(256)
    sfcKeysBatchKernel(const T* __restrict__ x, const T* __restrict__ y, const T* __restrict__ z,
                       const T* __restrict__ h, size_t n, const uint32_t* __restrict__ setOffsets, int numSets,
                       const KeyParams<T, uint32_t>* __restrict__ kps, uint64_t* __restrict__ keys,
                       PackedT<T>* __restrict__ packed)
{
    __shared__ uint16_t sH[384];
    const uint16_t* ht = stageHilbertTable<Kind>(sH);
    size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    {
        // the set holding particle i: last s with setOffsets[s] <= i
        int lo = 0, hi = numSets;
        while (lo + 1 < hi)
        {
            int mid = (lo + hi) >> 1;
            if (__ldg(setOffsets + mid) <= i) lo = mid;
            else hi = mid;
        }
        T px = __ldcs(x + i), py = __ldcs(y + i), pz = __ldcs(z + i), ph = __ldcs(h + i);
        uint32_t k = sfc3D<T, uint32_t>(px, py, pz, kps[lo], Kind, ht);
        keys[i]    = (uint64_t(lo) << 30) | uint64_t(k);
        PackedT<T> r;
        r.x       = px;
        r.y       = py;
        r.z       = pz;
        r.w       = ph;
        packed[i] = r;
    }
}

template<class T>
int sfcKeysBatched(cudaStream_t s, const T* x, const T* y, const T* z, const T* h, size_t n, const uint32_t* setOffsets,
                   int numSets, const KeyParams<T, uint32_t>* kps, int kind, uint64_t* keys, PackedT<T>* packed)
{
    if (n == 0) return CS_OK;
    unsigned thr  = 256;
    size_t blocks = (n + thr - 1) / thr;
    unsigned grid = unsigned(blocks < size_t(smCount()) * 16 ? blocks : size_t(smCount()) * 16);
    if (kind == CS_HILBERT)
        sfcKeysBatchKernel<T, CS_HILBERT><<<grid, thr, 0, s>>>(x, y, z, h, n, setOffsets, numSets, kps, keys, packed);
    else
        sfcKeysBatchKernel<T, CS_MORTON><<<grid, thr, 0, s>>>(x, y, z, h, n, setOffsets, numSets, kps, keys, packed);
    CSG_CHECK_LAUNCH();
    return CS_OK;
}

template int sfcKeysBatched<float>(cudaStream_t, const float*, const float*, const float*, const float*, size_t,
                                   const uint32_t*, int, const KeyParams<float, uint32_t>*, int, uint64_t*, float4*);
template int sfcKeysBatched<double>(cudaStream_t, const double*, const double*, const double*, const double*, size_t,
                                    const uint32_t*, int, const KeyParams<double, uint32_t>*, int, uint64_t*,
                                    double4_32a*);

template<class T, bool Shadow>
__global__ void __launch_bounds__(256) gatherPackedKernel(const uint32_t* __restrict__ perm, size_t n,
                                                          const PackedT<T>* __restrict__ packed, T* __restrict__ xs,
                                                          T* __restrict__ ys, T* __restrict__ zs, T* __restrict__ hs,
                                                          float4* __restrict__ phi, float4* __restrict__ plo,
                                                          float* cmax)
{
    size_t stride = size_t(gridDim.x) * blockDim.x;
    float m       = 0.f;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    {
        // an index past the end (a permutation from a sort that gave up) is clamped, so nothing is read out of range
        PackedT<T> r = packed[min(__ldcs(perm + i), uint32_t(n - 1))];
        __stcs(xs + i, r.x);
        __stcs(ys + i, r.y);
        __stcs(zs + i, r.z);
        __stcs(hs + i, r.w);
        if constexpr (Shadow)
        {
            // x = hi + lo to about 2^-48 relative; hi is x rounded to float
            float h0, h1, h2, l0, l1, l2;
            splitDouble(r.x, h0, l0);
            splitDouble(r.y, h1, l1);
            splitDouble(r.z, h2, l2);
            phi[i]   = make_float4(h0, h1, h2, 0.f);
            plo[i]   = make_float4(l0, l1, l2, 0.f);
            m        = fmaxf(m, fmaxf(fabsf(h0), fmaxf(fabsf(h1), fabsf(h2))));
        }
    }
    if constexpr (Shadow)
    {
        for (int o = 16; o > 0; o >>= 1)
            m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if ((threadIdx.x & 31) == 0 && m > 0.f) atomicMax(reinterpret_cast<int*>(cmax), __float_as_int(m));
    }
}

template<class T>
int gatherPacked(cudaStream_t s, const uint32_t* perm, size_t n, const PackedT<T>* packed, T* xs, T* ys, T* zs,
                 T* hs, float4* phi, float4* plo, float* cmax)
{
    if (n == 0) return CS_OK;
    unsigned thr  = 256;
    size_t blocks = (n + thr - 1) / thr;
    unsigned grid = unsigned(blocks < size_t(smCount()) * 32 ? blocks : size_t(smCount()) * 32);
    if constexpr (std::is_same_v<T, double>)
    {
        if (phi)
        {
            gatherPackedKernel<T, true><<<grid, thr, 0, s>>>(perm, n, packed, xs, ys, zs, hs, phi, plo, cmax);
            CSG_CHECK_LAUNCH();
            return CS_OK;
        }
    }
    gatherPackedKernel<T, false><<<grid, thr, 0, s>>>(perm, n, packed, xs, ys, zs, hs, phi, plo, cmax);
    CSG_CHECK_LAUNCH();
    return CS_OK;
}

template int gatherPacked<float>(cudaStream_t, const uint32_t*, size_t, const float4*, float*, float*, float*, float*,
                                 float4*, float4*, float*);
template int gatherPacked<double>(cudaStream_t, const uint32_t*, size_t, const double4_32a*, double*, double*,
                                  double*, double*, float4*, float4*, float*);

// ---------------------------------------------------------------------------------------------------------------
// gathers: out[i] = in[perm[i]]. The permutation is read once for up to four arrays.
// ---------------------------------------------------------------------------------------------------------------
template<class T, int NA>
__global__ void __launch_bounds__(256) gatherKernel(const uint32_t* __restrict__ perm, size_t n,
                                                    GatherArgs<T, NA> a)
{
    size_t stride = size_t(gridDim.x) * blockDim.x;
    for (size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    {
        uint32_t j = __ldcs(perm + i);
#pragma unroll
        for (int k = 0; k < NA; ++k)
            __stcs(a.out[k] + i, __ldg(a.in[k] + j));
    }
}

template<class T, int NA>
int gatherN(cudaStream_t s, const uint32_t* perm, size_t n, GatherArgs<T, NA> a)
{
    if (n == 0) return CS_OK;
    unsigned thr  = 256;
    size_t blocks = (n + thr - 1) / thr;
    unsigned grid = unsigned(blocks < size_t(smCount()) * 32 ? blocks : size_t(smCount()) * 32);
    gatherKernel<T, NA><<<grid, thr, 0, s>>>(perm, n, a);
    CSG_CHECK_LAUNCH();
    return CS_OK;
}

template int gatherN(cudaStream_t, const uint32_t*, size_t, GatherArgs<float, 1>);
template int gatherN(cudaStream_t, const uint32_t*, size_t, GatherArgs<double, 1>);
template int gatherN(cudaStream_t, const uint32_t*, size_t, GatherArgs<float, 4>);
template int gatherN(cudaStream_t, const uint32_t*, size_t, GatherArgs<double, 4>);

} // namespace csg

using namespace csg;

#define CS_KEYS_ENTRY(kindname, KIND, kb, K, tb, T)                                                                    \
    extern "C" int cs_sfc_keys_##kindname##_##kb##_##tb(cs_stream_t stream, const T* x, const T* y, const T* z,        \
                                                         K* keys, size_t n, const cs_box* box, int respect)            \
    {                                                                                                                  \
        if (!box)                                                                                                      \
        {                                                                                                              \
            setLastError("sfc keys: null box");                                                                        \
            return CS_ERR_INVALID;                                                                                     \
        }                                                                                                              \
        return sfcKeys<T, K>(cudaStream_t(stream), x, y, z, keys, n, *box, KIND, respect != 0);                       \
    }

CS_KEYS_ENTRY(hilbert, CS_HILBERT, u32, uint32_t, f32, float)
CS_KEYS_ENTRY(hilbert, CS_HILBERT, u32, uint32_t, f64, double)
CS_KEYS_ENTRY(hilbert, CS_HILBERT, u64, uint64_t, f32, float)
CS_KEYS_ENTRY(hilbert, CS_HILBERT, u64, uint64_t, f64, double)
CS_KEYS_ENTRY(morton, CS_MORTON, u32, uint32_t, f32, float)
CS_KEYS_ENTRY(morton, CS_MORTON, u32, uint32_t, f64, double)
CS_KEYS_ENTRY(morton, CS_MORTON, u64, uint64_t, f32, float)
CS_KEYS_ENTRY(morton, CS_MORTON, u64, uint64_t, f64, double)

extern "C" int cs_gather_f32(cs_stream_t stream, const uint32_t* perm, const float* in, float* out, size_t n)
{
    GatherArgs<float, 1> a{{in}, {out}};
    return gatherN<float, 1>(cudaStream_t(stream), perm, n, a);
}
extern "C" int cs_gather_f64(cs_stream_t stream, const uint32_t* perm, const double* in, double* out, size_t n)
{
    GatherArgs<double, 1> a{{in}, {out}};
    return gatherN<double, 1>(cudaStream_t(stream), perm, n, a);
}
extern "C" int cs_gather4_f64(cs_stream_t stream, const uint32_t* perm, size_t n, const double* in0, const double* in1,
                              const double* in2, const double* in3, double* out0, double* out1, double* out2,
                              double* out3)
{
    GatherArgs<double, 4> a{{in0, in1, in2, in3}, {out0, out1, out2, out3}};
    return gatherN<double, 4>(cudaStream_t(stream), perm, n, a);
}
extern "C" int cs_gather4_f32(cs_stream_t stream, const uint32_t* perm, size_t n, const float* in0, const float* in1,
                              const float* in2, const float* in3, float* out0, float* out1, float* out2, float* out3)
{
    GatherArgs<float, 4> a{{in0, in1, in2, in3}, {out0, out1, out2, out3}};
    return gatherN<float, 4>(cudaStream_t(stream), perm, n, a);
}

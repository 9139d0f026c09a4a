// Internal interface of sfc_keys.cu (keys and gathers), used by the pipeline drivers.
#pragma once
#include "cs_common.cuh"

namespace csg
{

template<class T, class K>
int sfcKeys(cudaStream_t s, const T* x, const T* y, const T* z, K* keys, size_t n, const cs_box& box, int kind,
            bool respectRemove);

template<class T, int NA>
struct GatherArgs
{
    const T* in[NA];
    T* out[NA];
};

template<class T, int NA>
int gatherN(cudaStream_t s, const uint32_t* perm, size_t n, GatherArgs<T, NA> a);

//! x, y, z, h of one particle in one aligned record (one 32-byte sector for double)
template<class T>
struct Packed;
template<>
struct Packed<float>
{
    using type = float4;
};
template<>
struct Packed<double>
{
    using type = double4_32a;
};
template<class T>
using PackedT = typename Packed<T>::type;

//! many independent sets: set s holds input particles [setOffsets[s], setOffsets[s + 1]) and its own box (kps[s]);
//! keys[i] = (s << 30) | the set's 32-bit key of particle i, so one sort of the combined keys sorts every set by its
//! own key and keeps the sets apart; the particles are packed as in sfcKeysPacked
template<class T>
int sfcKeysBatched(cudaStream_t s, const T* x, const T* y, const T* z, const T* h, size_t n, const uint32_t* setOffsets,
                   int numSets, const KeyParams<T, uint32_t>* kps, int kind, uint64_t* keys, PackedT<T>* packed);

//! keys as sfcKeys (no removeKey entries), and the particles packed into one record each
template<class T, class K>
int sfcKeysPacked(cudaStream_t s, const T* x, const T* y, const T* z, const T* h, K* keys, PackedT<T>* packed,
                  size_t n, const cs_box& box, int kind);

//! out[i] = packed[perm[i]] split into x, y, z, h; for T = double also the float shadows x = hi + lo of the
//! neighbour search and the running bound cmax (an atomic max over |hi|, not reset here)
template<class T>
int gatherPacked(cudaStream_t s, const uint32_t* perm, size_t n, const PackedT<T>* packed, T* xs, T* ys, T* zs,
                 T* hs, float4* phi, float4* plo, float* cmax);

} // namespace csg

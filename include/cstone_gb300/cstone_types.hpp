// The cstone interface types the GB300 shim needs, for builds without the reference's headers
// (CSTONE_GB300_STANDALONE). Member names, layouts and constructor arguments follow the reference's types, so code
// written against them compiles unchanged; only what the shim and its callers use is defined:
//
//   TreeNodeIndex, LocalIndex              tree/definitions.h
//   util::array, Vec3                      util/array.hpp
//   BoundaryType, Box<T>                   sfc/box.hpp:77-175 (lengths and inverse lengths in T, as there)
//   MortonKey<I>, HilbertKey<I>            sfc/sfc.hpp:31-114 (strong key types)
//   maxTreeLevel, nodeRange                sfc/common.hpp
//   execution::Gpu, gpuStream              execution.hpp:37-56
//   OctreeView, OctreeNsView               tree/octree.hpp:233-283
//   GroupView                              traversal/groups.hpp:28-34
//   DeviceVector, rawPtr, nNodes           cuda/device_vector.h (a minimal stream-less device vector)
#pragma once

#include <cstddef>
#include <cstdint>
#include <span>
#include <stdexcept>
#include <type_traits>
#include <utility>

#include <cuda_runtime.h>

#ifndef HOST_DEVICE_FUN
#define HOST_DEVICE_FUN __host__ __device__
#endif

namespace cstone
{

using TreeNodeIndex = int;
using LocalIndex    = unsigned;

namespace util
{
template<class T, std::size_t N>
struct array
{
    T data_[N];
    HOST_DEVICE_FUN constexpr T& operator[](std::size_t i) { return data_[i]; }
    HOST_DEVICE_FUN constexpr const T& operator[](std::size_t i) const { return data_[i]; }
    HOST_DEVICE_FUN constexpr T* data() { return data_; }
    HOST_DEVICE_FUN constexpr const T* data() const { return data_; }
    static constexpr std::size_t size() { return N; }
};

template<class T, std::size_t N>
HOST_DEVICE_FUN constexpr array<T, N> operator-(const array<T, N>& a, const array<T, N>& b)
{
    array<T, N> r{};
    for (std::size_t k = 0; k < N; ++k)
        r[k] = a[k] - b[k];
    return r;
}
} // namespace util

template<class T>
using Vec3 = util::array<T, 3>;

template<class T>
HOST_DEVICE_FUN constexpr T norm2(const Vec3<T>& v)
{
    return v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
}

enum class BoundaryType : char
{
    open     = 0,
    periodic = 1,
    fixed    = 2,
};

template<class T>
class Box
{
public:
    HOST_DEVICE_FUN constexpr Box(T xyzMin, T xyzMax, BoundaryType b = BoundaryType::open)
        : Box(xyzMin, xyzMax, xyzMin, xyzMax, xyzMin, xyzMax, b, b, b)
    {
    }
    HOST_DEVICE_FUN constexpr Box(T xmin, T xmax, T ymin, T ymax, T zmin, T zmax, BoundaryType bx = BoundaryType::open,
                                  BoundaryType by = BoundaryType::open, BoundaryType bz = BoundaryType::open)
        : limits_{xmin, xmax, ymin, ymax, zmin, zmax}
        , lengths_{xmax - xmin, ymax - ymin, zmax - zmin}
        , inverseLengths_{T(1) / (xmax - xmin), T(1) / (ymax - ymin), T(1) / (zmax - zmin)}
        , boundaries_{bx, by, bz}
    {
    }
    HOST_DEVICE_FUN constexpr T xmin() const { return limits_[0]; }
    HOST_DEVICE_FUN constexpr T xmax() const { return limits_[1]; }
    HOST_DEVICE_FUN constexpr T ymin() const { return limits_[2]; }
    HOST_DEVICE_FUN constexpr T ymax() const { return limits_[3]; }
    HOST_DEVICE_FUN constexpr T zmin() const { return limits_[4]; }
    HOST_DEVICE_FUN constexpr T zmax() const { return limits_[5]; }
    HOST_DEVICE_FUN constexpr T lx() const { return lengths_[0]; }
    HOST_DEVICE_FUN constexpr T ly() const { return lengths_[1]; }
    HOST_DEVICE_FUN constexpr T lz() const { return lengths_[2]; }
    HOST_DEVICE_FUN constexpr T ilx() const { return inverseLengths_[0]; }
    HOST_DEVICE_FUN constexpr T ily() const { return inverseLengths_[1]; }
    HOST_DEVICE_FUN constexpr T ilz() const { return inverseLengths_[2]; }
    HOST_DEVICE_FUN constexpr BoundaryType boundaryX() const { return boundaries_[0]; }
    HOST_DEVICE_FUN constexpr BoundaryType boundaryY() const { return boundaries_[1]; }
    HOST_DEVICE_FUN constexpr BoundaryType boundaryZ() const { return boundaries_[2]; }
    HOST_DEVICE_FUN constexpr T minExtent() const
    {
        T m = lengths_[0] < lengths_[1] ? lengths_[0] : lengths_[1];
        return m < lengths_[2] ? m : lengths_[2];
    }

private:
    T limits_[6];
    T lengths_[3];
    T inverseLengths_[3];
    BoundaryType boundaries_[3];
};

template<class I>
struct MortonKey
{
    using ValueType = I;
    I value;
};
template<class I>
struct HilbertKey
{
    using ValueType = I;
    I value;
};

template<class KeyType>
struct maxTreeLevel : std::integral_constant<unsigned, sizeof(KeyType) == 4 ? 10u : 21u>
{
};

template<class KeyType>
HOST_DEVICE_FUN constexpr KeyType nodeRange(unsigned level)
{
    return KeyType(1) << (3u * (maxTreeLevel<KeyType>{} - level));
}

namespace execution
{
struct Gpu
{
    operator cudaStream_t() const { return stream; }

private:
    constexpr explicit Gpu(cudaStream_t s) noexcept
        : stream(s)
    {
    }
    friend constexpr Gpu gpuStream(cudaStream_t s) noexcept;
    cudaStream_t stream;
};
constexpr inline Gpu gpuStream(cudaStream_t s) noexcept { return Gpu(s); }
} // namespace execution

template<class KeyType>
struct OctreeView
{
    using NodeType = std::conditional_t<std::is_const_v<KeyType>, const TreeNodeIndex, TreeNodeIndex>;
    TreeNodeIndex numLeafNodes;
    TreeNodeIndex numInternalNodes;
    TreeNodeIndex numNodes;
    TreeNodeIndex numParents;

    KeyType* prefixes;
    NodeType* childOffsets;
    NodeType* parents;
    NodeType* levelRange;
    NodeType* d_levelRange;
    NodeType* internalToLeaf;
    NodeType* leafToInternal;
    KeyType* leaves{nullptr};
};

template<class T, class KeyType>
struct OctreeNsView
{
    TreeNodeIndex numLeafNodes;
    TreeNodeIndex numNodes;
    const KeyType* prefixes;
    const TreeNodeIndex* childOffsets;
    const TreeNodeIndex* parents;
    const TreeNodeIndex* internalToLeaf;
    const TreeNodeIndex* leafToInternal;
    const TreeNodeIndex* levelRange;
    const KeyType* leaves;
    const LocalIndex* layout;
    const Vec3<T>* centers;
    const Vec3<T>* sizes;
    float searchExtFactor{1.0};
};

struct GroupView
{
    LocalIndex firstBody, lastBody;
    LocalIndex numGroups;
    const LocalIndex* groupStart;
    const LocalIndex* groupEnd;
};

//! device memory of n elements of T; resize keeps the first min(old, new) elements
template<class T>
class DeviceVector
{
public:
    using value_type = T;
    DeviceVector() = default;
    explicit DeviceVector(std::size_t n) { resize(n); }
    DeviceVector(const DeviceVector&)            = delete;
    DeviceVector& operator=(const DeviceVector&) = delete;
    DeviceVector(DeviceVector&& o) noexcept { swap(o); }
    DeviceVector& operator=(DeviceVector&& o) noexcept
    {
        swap(o);
        return *this;
    }
    ~DeviceVector()
    {
        if (ptr_) cudaFree(ptr_);
    }
    void resize(std::size_t n)
    {
        if (n <= cap_)
        {
            size_ = n;
            return;
        }
        T* p = nullptr;
        if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess) throw std::runtime_error("DeviceVector: cudaMalloc failed");
        if (ptr_ && size_) cudaMemcpy(p, ptr_, size_ * sizeof(T), cudaMemcpyDeviceToDevice);
        if (ptr_) cudaFree(ptr_);
        ptr_  = p;
        size_ = cap_ = n;
    }
    std::size_t size() const { return size_; }
    T* data() { return ptr_; }
    const T* data() const { return ptr_; }
    void swap(DeviceVector& o) noexcept
    {
        std::swap(ptr_, o.ptr_);
        std::swap(size_, o.size_);
        std::swap(cap_, o.cap_);
    }

private:
    T* ptr_          = nullptr;
    std::size_t size_ = 0, cap_ = 0;
};

template<class T>
void swap(DeviceVector<T>& a, DeviceVector<T>& b) noexcept
{
    a.swap(b);
}
template<class T>
T* rawPtr(DeviceVector<T>& v)
{
    return v.data();
}
template<class T>
const T* rawPtr(const DeviceVector<T>& v)
{
    return v.data();
}
template<class V>
TreeNodeIndex nNodes(const V& tree)
{
    return TreeNodeIndex(tree.size()) - 1;
}

} // namespace cstone

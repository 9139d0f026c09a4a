// A neighbourhood builder with the reference's ijLoop interface (traversal/ijloop/ijloop.hpp:120-146) over the GB300
// cluster-pair lists of libcstone_gb300 (cs_cluster_nblist_build_*). Compile with nvcc; include after
// cstone_gb300/cstone_gpu_shim.hpp (which brings in the reference's types, or their restatement with
// CSTONE_GB300_STANDALONE).
//
//   auto nb = cstone::ijloop::Gb300ClusterNeighborhoodBuilder{ncmax}.build(exec, treeView, box, totalBodies, groups,
//                                                                         x, y, z, h);
//   nb.ijLoop(std::tuple(m), std::tuple(rho), interaction, postamble);
//
// build() makes the cluster lists for all totalBodies particles (clusters of 8 consecutive particles; every j within
// 2 h_i of a particle i of an i-cluster is in one of its listed j-clusters). ijLoop() runs, for every target i in
// [groups.firstBody, groups.lastBody), result = interaction(iData, iData, 0, 0), then adds
// interaction(iData, jData, x_i - x_j, |x_i - x_j|^2) for every j != i with |x_i - x_j|^2 < (2 h_i)^2 in ascending j
// (as the reference's loops, traversal/ijloop/common.hpp and cpu_fullnblist.hpp:94-112), and stores
// postamble(iData, result) into the outputs at i. iData/jData are tuples (index, Vec3 position, h, inputs...) as in
// the reference. Open boxes; sum reductions (the reference's min/max/symmetric result modifiers are not provided).
// h may be a pointer (same type as the coordinates, or float with double coordinates) or a constant.
#pragma once

#include <cstdint>
#include <stdexcept>
#include <tuple>
#include <type_traits>
#include <utility>

#include <cuda_runtime.h>

#include "cstone_gb300.h"
#ifndef CSTONE_GB300_STANDALONE
#include "cstone/traversal/ijloop/ijloop.hpp" // Statistics, empty_postamble, GroupView
#endif

namespace cstone::ijloop
{

#ifdef CSTONE_GB300_STANDALONE
struct Statistics
{
    const std::size_t numBodies, numBytes;
};
namespace detail
{
struct EmptyPostamble
{
    template<class P, class R>
    __host__ __device__ constexpr R operator()(P const&, R const& r) const
    {
        return r;
    }
};
} // namespace detail
constexpr detail::EmptyPostamble empty_postamble;
#endif

namespace gb300_detail
{

template<class T>
__device__ __forceinline__ T loadOne(const T* p, LocalIndex i)
{
    return __ldg(p + i);
}

template<class Tc, class Th, class... In>
__device__ __forceinline__ auto particleData(const Tc* x, const Tc* y, const Tc* z, const Th* h,
                                             const std::tuple<const In*...>& in, LocalIndex i)
{
    Vec3<Tc> pos{loadOne(x, i), loadOne(y, i), loadOne(z, i)};
    return std::tuple_cat(std::make_tuple(i, pos, loadOne(h, i)),
                          std::apply([i](auto const*... p) { return std::make_tuple(loadOne(p, i)...); }, in));
}

template<class... Ts, std::size_t... I>
__device__ __forceinline__ void addTuple(std::tuple<Ts...>& r, const std::tuple<Ts...>& v, std::index_sequence<I...>)
{
    ((std::get<I>(r) += std::get<I>(v)), ...);
}

template<class... Out, class... Ts, std::size_t... I>
__device__ __forceinline__ void storeTuple(const std::tuple<Out*...>& out, LocalIndex i, const std::tuple<Ts...>& v,
                                           std::index_sequence<I...>)
{
    ((std::get<I>(out)[i] = std::get<I>(v)), ...);
}

constexpr int CL = 8;

template<class Tc, class Th, class InT, class OutT, class Interaction, class Postamble>
__global__ void clusterIjLoopKernel(const Tc* x, const Tc* y, const Tc* z, const Th* h, InT in, OutT out,
                                    Interaction interaction, Postamble postamble, LocalIndex firstBody,
                                    LocalIndex lastBody, std::size_t n, const uint32_t* lists,
                                    const uint32_t* counts, unsigned ncmax)
{
    const LocalIndex i = firstBody + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= lastBody) return;
    const auto iData = particleData(x, y, z, h, in, i);
    // radiusSq = 4 h h in the precision of h (traversal/ijloop/common.hpp:176-181)
    const Th r2h     = Th(4) * std::get<2>(iData) * std::get<2>(iData);
    auto result      = interaction(iData, iData, Vec3<Tc>{0, 0, 0}, Tc(0));
    const LocalIndex ic = i / CL;
    const unsigned cnt  = min(counts[ic], ncmax);
    const uint32_t* row = lists + std::size_t(ic) * ncmax;
    for (unsigned t = 0; t < cnt; ++t)
    {
        const std::size_t J = row[t];
        for (int q = 0; q < CL; ++q)
        {
            const std::size_t j = J * CL + q;
            if (j >= n || j == i) continue;
            const auto jData = particleData(x, y, z, h, in, LocalIndex(j));
            const Vec3<Tc> d{std::get<1>(iData)[0] - std::get<1>(jData)[0],
                             std::get<1>(iData)[1] - std::get<1>(jData)[1],
                             std::get<1>(iData)[2] - std::get<1>(jData)[2]};
            const Tc d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            if (d2 < r2h)
                addTuple(result, interaction(iData, jData, d, d2),
                         std::make_index_sequence<std::tuple_size_v<decltype(result)>>{});
        }
    }
    const auto final = postamble(iData, result);
    storeTuple(out, i, final, std::make_index_sequence<std::tuple_size_v<std::decay_t<decltype(final)>>>{});
}

template<class Tc, class Th>
__global__ void fillKernel(Tc* dst, const Th* src, Th value, std::size_t n)
{
    std::size_t k = std::size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k < n) dst[k] = src ? Tc(src[k]) : Tc(value);
}

inline void check(int rc, const char* what)
{
    if (rc != CS_OK) throw std::runtime_error(std::string(what) + ": " + cs_last_error());
}

} // namespace gb300_detail

template<class Tc, class ThP>
struct Gb300ClusterNeighborhood
{
    using Th = std::remove_cvref_t<std::remove_pointer_t<ThP>>;
    cudaStream_t stream  = nullptr;
    LocalIndex firstBody = 0, lastBody = 0;
    std::size_t totalBodies = 0;
    const Tc *x = nullptr, *y = nullptr, *z = nullptr;
    const Th* h = nullptr; // device h of every particle (a constant h is stored per particle)
    uint32_t* lists  = nullptr;
    uint32_t* counts = nullptr;
    Th* hOwned       = nullptr;
    unsigned ncmax   = 0;

    Gb300ClusterNeighborhood() = default;
    Gb300ClusterNeighborhood(const Gb300ClusterNeighborhood&) = delete;
    Gb300ClusterNeighborhood(Gb300ClusterNeighborhood&& o) noexcept { *this = std::move(o); }
    Gb300ClusterNeighborhood& operator=(Gb300ClusterNeighborhood&& o) noexcept
    {
        std::swap(stream, o.stream), std::swap(firstBody, o.firstBody), std::swap(lastBody, o.lastBody);
        std::swap(totalBodies, o.totalBodies), std::swap(x, o.x), std::swap(y, o.y), std::swap(z, o.z);
        std::swap(h, o.h), std::swap(lists, o.lists), std::swap(counts, o.counts), std::swap(hOwned, o.hOwned);
        std::swap(ncmax, o.ncmax);
        return *this;
    }
    ~Gb300ClusterNeighborhood()
    {
        if (lists) cudaFree(lists);
        if (counts) cudaFree(counts);
        if (hOwned) cudaFree(hOwned);
    }

    template<class... In, class... Out, class Interaction, class Postamble>
    void ijLoop(std::tuple<In*...> const& input, std::tuple<Out*...> const& output, Interaction&& interaction,
                Postamble&& postamble) const
    {
        if (lastBody <= firstBody) return;
        std::tuple<const In*...> cin = std::apply([](auto*... p) { return std::tuple<const In*...>(p...); }, input);
        unsigned blocks = unsigned((lastBody - firstBody + 127) / 128);
        gb300_detail::clusterIjLoopKernel<<<blocks, 128, 0, stream>>>(
            x, y, z, h, cin, output, std::decay_t<Interaction>(interaction), std::decay_t<Postamble>(postamble),
            firstBody, lastBody, totalBodies, lists, counts, ncmax);
        if (cudaGetLastError() != cudaSuccess) throw std::runtime_error("ijLoop: kernel launch failed");
    }

    Statistics stats() const
    {
        return {std::size_t(lastBody - firstBody), ((totalBodies + 7) / 8) * (std::size_t(ncmax) + 1) * 4};
    }
};

//! NeighborhoodBuilder over the cluster lists: ncmax j-clusters per i-cluster (grown to what is needed)
struct Gb300ClusterNeighborhoodBuilder
{
    unsigned ncmax = 256;

    template<class Tc, class KeyType, class ThP>
    Gb300ClusterNeighborhood<Tc, ThP> build(execution::Gpu exec, const OctreeNsView<Tc, KeyType>& tree,
                                            const Box<Tc>& box, LocalIndex totalBodies, const GroupView& groups,
                                            const Tc* x, const Tc* y, const Tc* z, ThP h) const
    {
        using Th = typename Gb300ClusterNeighborhood<Tc, ThP>::Th;
        static_assert(std::is_same_v<Tc, double> || std::is_same_v<Tc, float>, "float or double coordinates");
        Gb300ClusterNeighborhood<Tc, ThP> nb;
        nb.stream      = static_cast<cudaStream_t>(exec);
        nb.firstBody   = groups.firstBody;
        nb.lastBody    = groups.lastBody;
        nb.totalBodies = totalBodies;
        nb.x = x, nb.y = y, nb.z = z;
        if (totalBodies == 0) return nb;
        // the cluster build reads h in the coordinate type
        Tc* hc = nullptr;
        if (cudaMallocAsync(&hc, totalBodies * sizeof(Tc), nb.stream) != cudaSuccess)
            throw std::runtime_error("cluster lists: cudaMallocAsync failed");
        const Th* hp = nullptr;
        Th hv{};
        if constexpr (std::is_pointer_v<ThP>) hp = h;
        else hv = h;
        gb300_detail::fillKernel<<<unsigned((totalBodies + 255) / 256), 256, 0, nb.stream>>>(hc, hp, hv,
                                                                                            std::size_t(totalBodies));
        if constexpr (std::is_pointer_v<ThP>) nb.h = h;
        else
        {
            if (cudaMallocAsync(&nb.hOwned, totalBodies * sizeof(Th), nb.stream) != cudaSuccess)
                throw std::runtime_error("cluster lists: cudaMallocAsync failed");
            gb300_detail::fillKernel<<<unsigned((totalBodies + 255) / 256), 256, 0, nb.stream>>>(
                nb.hOwned, static_cast<const Th*>(nullptr), hv, std::size_t(totalBodies));
            nb.h = nb.hOwned;
        }
        cs_box cb;
        cb.lo[0] = double(box.xmin()), cb.lo[1] = double(box.ymin()), cb.lo[2] = double(box.zmin());
        cb.hi[0] = double(box.xmax()), cb.hi[1] = double(box.ymax()), cb.hi[2] = double(box.zmax());
        cb.boundary[0] = int(box.boundaryX()), cb.boundary[1] = int(box.boundaryY());
        cb.boundary[2] = int(box.boundaryZ());
        cs_ns_view v{tree.numLeafNodes, tree.numNodes, tree.childOffsets, tree.parents, tree.internalToLeaf,
                     tree.layout,       tree.centers,  tree.sizes,        tree.searchExtFactor};
        const std::size_t nic = (std::size_t(totalBodies) + 7) / 8;
        unsigned cap          = ncmax;
        for (;;)
        {
            if (cudaMalloc(&nb.lists, nic * cap * sizeof(uint32_t)) != cudaSuccess ||
                cudaMalloc(&nb.counts, nic * sizeof(uint32_t)) != cudaSuccess)
                throw std::runtime_error("cluster lists: cudaMalloc failed");
            int mx = 0, rc;
            if constexpr (std::is_same_v<Tc, double>)
                rc = cs_cluster_nblist_build_f64(nb.stream, x, y, z, hc, totalBodies, &v, &cb, int(8 * sizeof(KeyType)),
                                                 cap, nb.lists, nb.counts, nullptr, 0, &mx);
            else
                rc = cs_cluster_nblist_build_f32(nb.stream, x, y, z, hc, totalBodies, &v, &cb, int(8 * sizeof(KeyType)),
                                                 cap, nb.lists, nb.counts, nullptr, 0, &mx);
            if (rc == CS_ERR_CAPACITY)
            {
                cudaFree(nb.lists), cudaFree(nb.counts);
                nb.lists = nb.counts = nullptr;
                cap                  = unsigned(mx);
                continue;
            }
            gb300_detail::check(rc, "cluster lists");
            break;
        }
        nb.ncmax = cap;
        cudaFreeAsync(hc, nb.stream);
        return nb;
    }
};

} // namespace cstone::ijloop

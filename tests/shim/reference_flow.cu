// A program written against the reference's GPU API (namespace cstone), run on libcstone_gb300 through the shim:
// the flow of the reference's GPU tests and benchmarks (test/unit_cuda/tree/csarray.cu:163-185 for the leaf array,
// test/performance/octree.cu for the rest): keys -> sortByKey -> gather -> updateOctreeGpu until converged ->
// buildOctreeGpu -> computeGeoCentersGpu -> computeBoundingBoxGpu -> findHalosGpu -> a NeighborhoodBuilder's
// build().ijLoop() with an SPH density interaction.
//
// Built two ways by tests/test_shim_flow.py: against the reference's headers (compile only, where they exist: the
// declarations check the shim) and with -DCSTONE_GB300_STANDALONE (no reference headers), run on the GPU.
//
// Usage: reference_flow <input file> <output directory>
//   input: int64 n, double lo[3], hi[3], int32 bucket, int32 focus leaves (first, last) selector unused (0),
//          then n doubles each of x, y, z, h, m
//   output files (raw arrays): keys, order, leaves, counts, prefixes, child_offsets, parents, centers, sizes,
//          flags, rho, plus meta.txt (leaves, nodes, iterations)
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "cstone_gb300/cstone_gpu_shim.hpp"
#include "cstone_gb300/ijloop_gb300.cuh"

#ifndef CSTONE_GB300_STANDALONE
#include "cstone/cuda/device_vector.h"
#include "cstone/tree/update_gpu.cuh"
// the builder satisfies the reference's own concept (traversal/ijloop/ijloop.hpp:120-146)
static_assert(cstone::ijloop::NeighborhoodBuilder<cstone::ijloop::Gb300ClusterNeighborhoodBuilder>);
#endif

using namespace cstone;

// the density interaction of the tests: m_j w(q), q = sqrt(d2) / h_i, w = (1 - 1.5 q^2) + (0.75 q^2) q for q < 1,
// else 0.25 ((2 - q)^2 (2 - q)); the postamble multiplies the sum by 1 / h_i^3
struct Density
{
    template<class I, class J, class V, class T>
    __device__ std::tuple<double> operator()(const I& iData, const J& jData, const V&, T d2) const
    {
        const double hinv = 1.0 / std::get<2>(iData);
        const double q    = sqrt(d2) * hinv;
        const double q2   = q * q;
        double w;
        if (q < 1.0) w = (1.0 - 1.5 * q2) + (0.75 * q2) * q;
        else
        {
            const double t = 2.0 - q;
            w              = 0.25 * ((t * t) * t);
        }
        return {std::get<3>(jData) * w};
    }
};

struct DensityPost
{
    template<class I>
    __device__ std::tuple<double> operator()(const I& iData, const std::tuple<double>& r) const
    {
        const double hinv = 1.0 / std::get<2>(iData);
        return {std::get<0>(r) * ((hinv * hinv) * hinv)};
    }
};

__global__ void iotaKernel(unsigned* v, size_t n)
{
    size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) v[i] = unsigned(i);
}

template<class V>
static void save(const std::string& path, const V& dev, size_t n)
{
    using T = std::remove_cv_t<std::remove_pointer_t<decltype(rawPtr(dev))>>;
    std::vector<T> h(n);
    if (n) cudaMemcpy(h.data(), rawPtr(dev), n * sizeof(T), cudaMemcpyDeviceToHost);
    std::ofstream f(path, std::ios::binary);
    f.write(reinterpret_cast<const char*>(h.data()), std::streamsize(n * sizeof(T)));
}

template<class T>
static void upload(DeviceVector<T>& d, const std::vector<T>& h)
{
    d.resize(h.size());
    cudaMemcpy(rawPtr(d), h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice);
}

int main(int argc, char** argv)
{
    if (argc < 3)
    {
        std::fprintf(stderr, "usage: %s input outdir\n", argv[0]);
        return 2;
    }
    using KeyType = uint64_t;
    using T       = double;
    std::ifstream in(argv[1], std::ios::binary);
    int64_t n64;
    double lo[3], hi[3];
    int32_t bucket, unused;
    in.read(reinterpret_cast<char*>(&n64), 8);
    in.read(reinterpret_cast<char*>(lo), 24);
    in.read(reinterpret_cast<char*>(hi), 24);
    in.read(reinterpret_cast<char*>(&bucket), 4);
    in.read(reinterpret_cast<char*>(&unused), 4);
    const size_t n = size_t(n64);
    std::vector<T> hx(n), hy(n), hz(n), hh(n), hm(n);
    for (auto* v : {&hx, &hy, &hz, &hh, &hm})
        in.read(reinterpret_cast<char*>(v->data()), std::streamsize(n * sizeof(T)));
    const std::string out = argv[2];

    auto exec = execution::gpuStream(0);
    Box<T> box(lo[0], hi[0], lo[1], hi[1], lo[2], hi[2]);

    DeviceVector<T> x, y, z, h, m, xs, ys, zs, hs, ms;
    upload(x, hx), upload(y, hy), upload(z, hz), upload(h, hh), upload(m, hm);
    for (auto* v : {&xs, &ys, &zs, &hs, &ms})
        v->resize(n);

    // keys and the stable sort with the ordering
    DeviceVector<KeyType> keys(n), keyBuf(n);
    DeviceVector<unsigned> order(n), orderBuf(n);
    computeSfcKeys(exec, rawPtr(x), rawPtr(y), rawPtr(z), reinterpret_cast<HilbertKey<KeyType>*>(rawPtr(keys)), n, box);
    iotaKernel<<<unsigned((n + 255) / 256), 256>>>(rawPtr(order), n);
    DeviceVector<char> tmp(sortByKeyTempStorage<KeyType, unsigned>(n));
    sortByKey(exec, rawPtr(keys), rawPtr(keys) + n, rawPtr(order), rawPtr(keyBuf), rawPtr(orderBuf), rawPtr(tmp),
              tmp.size());
    gather(exec, rawPtr(order), n, rawPtr(x), rawPtr(xs));
    gather(exec, rawPtr(order), n, rawPtr(y), rawPtr(ys));
    gather(exec, rawPtr(order), n, rawPtr(z), rawPtr(zs));
    gather(exec, rawPtr(order), n, rawPtr(h), rawPtr(hs));
    gather(exec, rawPtr(order), n, rawPtr(m), rawPtr(ms));

    // the cornerstone leaf array from the root, one updateOctreeGpu step at a time until converged
    DeviceVector<KeyType> tree, tmpTree;
    DeviceVector<unsigned> counts;
    DeviceVector<TreeNodeIndex> work;
    upload(tree, std::vector<KeyType>{0, nodeRange<KeyType>(0)});
    upload(counts, std::vector<unsigned>{unsigned(n)});
    std::span<const KeyType> keySpan(rawPtr(keys), n);
    int iterations = 0;
    while (!updateOctreeGpu(exec, keySpan, unsigned(bucket), tree, counts, tmpTree, work))
        ++iterations;
    ++iterations;
    const TreeNodeIndex L = nNodes(tree);

    // the internal tree
    const TreeNodeIndex I = (L - 1) / 7, N = L + I;
    DeviceVector<KeyType> prefixes(N);
    DeviceVector<TreeNodeIndex> childOffsets(N + 1), parents(std::max(1, (N - 1) / 8)), i2l(N), l2i(N),
        dLevelRange(maxTreeLevel<KeyType>{} + 2);
    std::vector<TreeNodeIndex> levelRange(maxTreeLevel<KeyType>{} + 2);
    OctreeView<KeyType> view{L,
                             I,
                             N,
                             TreeNodeIndex(std::max(1, (N - 1) / 8)),
                             rawPtr(prefixes),
                             rawPtr(childOffsets),
                             rawPtr(parents),
                             levelRange.data(),
                             rawPtr(dLevelRange),
                             rawPtr(i2l),
                             rawPtr(l2i)};
    buildOctreeGpu(exec, rawPtr(tree), view);

    DeviceVector<Vec3<T>> centers(N), sizes(N);
    computeGeoCentersGpu(exec, rawPtr(prefixes), N, rawPtr(centers), rawPtr(sizes), box);

    // particle layout of the leaves
    DeviceVector<unsigned> layout(L + 1);
    DeviceVector<unsigned> countsPlus(L + 1);
    cudaMemset(rawPtr(countsPlus), 0, (L + 1) * sizeof(unsigned));
    cudaMemcpy(rawPtr(countsPlus), rawPtr(counts), L * sizeof(unsigned), cudaMemcpyDeviceToDevice);
    exclusiveScan(exec, rawPtr(countsPlus), rawPtr(countsPlus) + L + 1, rawPtr(layout), 0u);

    // halos of the leaves in the first quarter of the key space: search boxes start from the leaves' centres
    std::vector<KeyType> hostTree(L + 1);
    cudaMemcpy(hostTree.data(), rawPtr(tree), (L + 1) * sizeof(KeyType), cudaMemcpyDeviceToHost);
    TreeNodeIndex first = 0, last = 0;
    while (last < L && hostTree[last] < nodeRange<KeyType>(0) / 4)
        ++last;
    std::vector<TreeNodeIndex> hl2i(N);
    cudaMemcpy(hl2i.data(), rawPtr(l2i), N * sizeof(TreeNodeIndex), cudaMemcpyDeviceToHost);
    std::vector<Vec3<T>> hcenters(N), hinit(L);
    cudaMemcpy(hcenters.data(), rawPtr(centers), N * sizeof(Vec3<T>), cudaMemcpyDeviceToHost);
    for (TreeNodeIndex l = 0; l < L; ++l)
        hinit[l] = hcenters[hl2i[I + l]];
    DeviceVector<Vec3<T>> searchCenters, searchSizes(L);
    upload(searchCenters, hinit);
    computeBoundingBoxGpu(exec, rawPtr(xs), rawPtr(ys), rawPtr(zs), rawPtr(hs), rawPtr(layout), first, last, T(2),
                          rawPtr(searchCenters), rawPtr(searchSizes));
    DeviceVector<uint8_t> flags(N);
    cudaMemset(rawPtr(flags), 0, N);
    findHalosGpu(exec, rawPtr(prefixes), rawPtr(childOffsets), rawPtr(parents), rawPtr(centers), rawPtr(sizes),
                 rawPtr(tree), rawPtr(searchCenters), rawPtr(searchSizes), box, first, last, rawPtr(flags));

    // neighbours through a NeighborhoodBuilder and an ijLoop
    OctreeNsView<T, KeyType> ns{L,       N,       rawPtr(prefixes), rawPtr(childOffsets), rawPtr(parents), rawPtr(i2l),
                                rawPtr(l2i), rawPtr(dLevelRange), rawPtr(tree), rawPtr(layout), rawPtr(centers),
                                rawPtr(sizes), 1.0f};
    GroupView groups{0, LocalIndex(n), 0, nullptr, nullptr};
    DeviceVector<double> rho(n);
    auto nb = ijloop::Gb300ClusterNeighborhoodBuilder{64}.build(exec, ns, box, LocalIndex(n), groups, rawPtr(xs),
                                                                rawPtr(ys), rawPtr(zs), (const T*)rawPtr(hs));
    nb.ijLoop(std::make_tuple(rawPtr(ms)), std::make_tuple(rawPtr(rho)), Density{}, DensityPost{});
    if (cudaDeviceSynchronize() != cudaSuccess)
    {
        std::fprintf(stderr, "CUDA error: %s\n", cudaGetErrorString(cudaGetLastError()));
        return 1;
    }

    save(out + "/keys", keys, n);
    save(out + "/order", order, n);
    save(out + "/leaves", tree, size_t(L) + 1);
    save(out + "/counts", counts, size_t(L));
    save(out + "/prefixes", prefixes, size_t(N));
    save(out + "/child_offsets", childOffsets, size_t(N));
    save(out + "/centers", centers, size_t(N));
    save(out + "/sizes", sizes, size_t(N));
    save(out + "/flags", flags, size_t(N));
    save(out + "/rho", rho, n);
    std::ofstream meta(out + "/meta.txt");
    meta << L << " " << N << " " << iterations << " " << first << " " << last << "\n";
    return 0;
}

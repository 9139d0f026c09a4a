// Internal interface of the neighbour search (neighbors.cu).
#pragma once
#include "cs_common.cuh"

namespace csg
{

template<class T>
struct NbArgs
{
    const T *x, *y, *z, *h;
    uint32_t first, last;
    BoxParams<T> b;
    int anyPbc;
    const int32_t* childOffsets;
    const int32_t* parents;
    const int32_t* i2l;
    const uint32_t* layout;
    const T* centers;
    const T* sizes;
    float ext;
    unsigned ngmax;
    uint32_t* nb;
    uint32_t* nc;
    //! optional traversal statistics (null: off): [0] lane cell tests, [1] cell tests decided in FP64,
    //! [2] lane pair tests, [3] pair tests decided in FP64, [4] leaves visited per warp, [5] candidates staged,
    //! [6] nodes visited per warp, [7] warps
    unsigned long long* stats = nullptr;
    //! path kernel: serve only warps that contain a particle whose search sphere crosses a periodic boundary
    int pathOnlyPbcWarps = 0;
    //! device error word (may be null): traversal stack overflow of the group kernel
    uint32_t* errWord = nullptr;
    //! smoothing lengths in float with coordinates of type T (then h is unused): the reference's findNeighbors with
    //! Tc = double, Th = float (radii rounded to float)
    const float* hf = nullptr;
    //! targets per warp of the group traversal (8, 16 or 32)
    int groupSize = 32;
    //! one target per lane (groupSize 32): a candidate batch runs the by-target loop when 19 x (needing lanes) is
    //! below byTargetCost x (candidate steps of the per-lane loop); 0 never. Speed only, results do not change
    int byTargetCost = 7;
    //! many independent sets in one tree (may be null): the sorted particles of set s are [setOffsets[s],
    //! setOffsets[s + 1]) and its traversal starts at node setRoots[s] instead of the root
    const uint32_t* setOffsets = nullptr;
    const int32_t* setRoots    = nullptr;
    int numSets                = 0;
};

//! float shadows for the FP64 pre-filter: particles x = hi + lo (two floats), and one record of three float4 per node
//!   nrec[3i]     centre rounded to float (hi),             w: child offset (int bits, 0 for a leaf)
//!   nrec[3i + 1] centre - hi rounded to float (lo),       w: first particle of a leaf (uint bits)
//!   nrec[3i + 2] half size rounded to nearest float,      w: end particle of a leaf (uint bits)
//! so that one broadcast load round gives a popped node's box, its children and its particle range
struct NbPrep
{
    const float4* phi  = nullptr;
    const float4* plo  = nullptr;
    const float4* nrec = nullptr;
    const float* cmax  = nullptr; // bound on |coordinate| over particles and node boxes
    //! per particle: 1 if it lies outside the box of its own leaf. The reference quantises a coordinate as
    //! int(floor(x * m) - xmin * m) (sfc/sfc.hpp:142-160), which can put a point into the finest cell below its
    //! geometric one, so near a leaf's upper faces a particle may lie outside its leaf's box by up to one finest
    //! cell. Such a candidate never takes the path-safe shortcut (it gets the exact ancestor walk).
    const uint8_t* pout = nullptr;
};

size_t nbPrepBytes(size_t n, int numNodes);

//! pout[j] for every particle of every leaf, and the marker (child offset -1) in the records of the leaves that hold
//! any outside particle; after the node records of prep are built. phi: the float shadows (T = double, may be null).
//! Launch over the nodes (Ldev: leaf count in device memory, numNodes then the capacity's node count)
template<class T>
int nbMarkOutside(cudaStream_t s, const T* x, const T* y, const T* z, const float4* phi, const T* centers,
                  const T* sizes, const int32_t* childOffsets, const int32_t* i2l, const uint32_t* layout,
                  int numNodes, const NbPrep& prep, uint8_t* pout, const int* Ldev = nullptr);
template<class T>
int nbPrepare(cudaStream_t s, const T* x, const T* y, const T* z, size_t n, const T* centers, const T* sizes,
              const int32_t* childOffsets, const int32_t* i2l, const uint32_t* layout, int numNodes, void* ws,
              size_t wsBytes, NbPrep* prep);

//! node part of nbPrepare only: the particle shadows (T = double) and cmax are set by the caller, cmax already holding
//! the particles' bound (the node boxes are folded in with an atomic max)
//! Ldev (may be null): the leaf count in device memory; numNodes is then the capacity's node count
template<class T>
int nbPrepareNodes(cudaStream_t s, const T* centers, const T* sizes, const int32_t* childOffsets,
                   const int32_t* i2l, const uint32_t* layout, int numNodes, void* ws, size_t wsBytes, NbPrep* prep,
                   const int* Ldev = nullptr);

template<class T>
NbArgs<T> makeNbArgs(const T* x, const T* y, const T* z, const T* h, uint32_t first, uint32_t last,
                     const cs_box& box, const cs_ns_view& v, unsigned ngmax, uint32_t* nb, uint32_t* nc);

template<class T>
int findNeighbors(cudaStream_t s, const NbArgs<T>& a, const NbPrep& prep);

} // namespace csg

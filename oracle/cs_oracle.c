/*
 * CPU restatement of the cornerstone-octree single-GPU path (oracle).
 *
 * TEST INFRASTRUCTURE ONLY: tests, the smoke check and the benchmark's CPU-baseline leg load this library as the
 * checker / CPU baseline. The CUDA product path never calls it.
 *
 * Build with -ffp-contract=off: the reference's arithmetic is evaluated without fused multiply-add (g++ on x86-64),
 * and every floating-point expression below keeps the reference's operation order.
 *
 * Parallel structure mirrors the reference's OpenMP CPU path: keys, counts, decisions, node processing, layout,
 * linking, geometry, halos and neighbours are `omp parallel for`; the stable key sort and the exclusive scans are
 * serial, as std::stable_sort and std::exclusive_scan are in the reference.
 */
#include "cs_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ------------------------------------------------------------------------------------------------------------ */
/* key algebra                                                                                                   */
/* ------------------------------------------------------------------------------------------------------------ */

static inline int max_level(int key_bits) { return key_bits == 32 ? 10 : 21; }

/* countLeadingZeros of a key of width key_bits (primitives/clz.hpp:65-108), 0 -> key_bits */
static inline int clzk(uint64_t x, int key_bits)
{
    if (x == 0) return key_bits;
    return __builtin_clzll(x) - (64 - key_bits);
}
static inline int unused_bits(int key_bits) { return key_bits == 32 ? 2 : 1; }

/* nodeRange (sfc/common.hpp:99-106) */
static inline uint64_t node_range(unsigned level, int key_bits)
{
    return (uint64_t)1 << (3u * (unsigned)(max_level(key_bits) - (int)level));
}
/* treeLevel (sfc/common.hpp:140-145) */
static inline unsigned tree_level(uint64_t range, int key_bits)
{
    return (unsigned)(clzk(range - 1, key_bits) - unused_bits(key_bits)) / 3u;
}
/* octalDigit (sfc/common.hpp:301-305) */
static inline unsigned octal_digit(uint64_t code, unsigned pos, int key_bits)
{
    return (unsigned)((code >> (3u * (unsigned)(max_level(key_bits) - (int)pos))) & 7u);
}
/* commonPrefix (sfc/common.hpp:127-131) */
static inline int common_prefix(uint64_t a, uint64_t b, int key_bits)
{
    return clzk(a ^ b, key_bits) - unused_bits(key_bits);
}
/* encodePlaceholderBit (sfc/common.hpp:172-180) */
static inline uint64_t encode_placeholder(uint64_t code, int prefix_length, int key_bits)
{
    int nshift = 3 * max_level(key_bits) - prefix_length;
    return ((uint64_t)1 << prefix_length) | (code >> nshift);
}
/* decodePrefixLength (sfc/common.hpp:190-194) */
static inline unsigned decode_prefix_length(uint64_t code) { return 63u - (unsigned)__builtin_clzll(code); }
/* decodePlaceholderBit (sfc/common.hpp:205-213) */
static inline uint64_t decode_placeholder(uint64_t code, int key_bits)
{
    unsigned len = decode_prefix_length(code);
    uint64_t ret = code ^ ((uint64_t)1 << len);
    return ret << (3u * (unsigned)max_level(key_bits) - len);
}
/* enclosingBoxCode (sfc/common.hpp:324-330) */
static inline uint64_t enclosing_box_code(uint64_t key, unsigned level, int key_bits)
{
    uint64_t mask = node_range(level, key_bits) - 1;
    return key & ~mask;
}
/* digitWeight (sfc/common.hpp:316-321) */
static inline int digit_weight(int digit)
{
    int four_geq_mask = -(int)(digit >= 4);
    return ((7 - digit) & four_geq_mask) - (digit & ~four_geq_mask);
}

/* Morton bit expansion (sfc/morton.hpp:35-72): every bit of the input is followed by two zero bits */
static uint64_t spread3(uint64_t v, int nbits)
{
    uint64_t r = 0;
    for (int b = 0; b < nbits; ++b)
        r |= ((v >> b) & 1u) << (3 * b);
    return r;
}
static unsigned compact3(uint64_t v, int nbits)
{
    unsigned r = 0;
    for (int b = 0; b < nbits; ++b)
        r |= (unsigned)((v >> (3 * b)) & 1u) << b;
    return r;
}

/* iMorton (sfc/morton.hpp:94-108): x bits go to position 3b+2, y to 3b+1, z to 3b */
uint64_t cso_imorton(unsigned ix, unsigned iy, unsigned iz, int key_bits)
{
    int L = max_level(key_bits);
    return spread3(ix, L) * 4 + spread3(iy, L) * 2 + spread3(iz, L);
}

void cso_decode_morton(uint64_t key, int key_bits, unsigned* ixyz)
{
    int L    = max_level(key_bits);
    ixyz[0] = compact3(key >> 2, L);
    ixyz[1] = compact3(key >> 1, L);
    ixyz[2] = compact3(key, L);
}

/* iHilbert (sfc/hilbert.hpp:43-94): one octant per level, most significant first. The octant of the rotated
 * coordinates is mapped through the Morton->Hilbert table {0,1,3,2,7,6,4,5}; then the remaining lower bits are
 * complemented and permuted according to the octant, as the reference's state update does. */
uint64_t cso_ihilbert(unsigned px, unsigned py, unsigned pz, int key_bits)
{
    static const unsigned m2h[8] = {0, 1, 3, 2, 7, 6, 4, 5};
    uint64_t key                 = 0;
    for (int level = max_level(key_bits) - 1; level >= 0; --level)
    {
        unsigned xi = (px >> level) & 1u;
        unsigned yi = (py >> level) & 1u;
        unsigned zi = (pz >> level) & 1u;
        key         = (key << 3) + m2h[(xi << 2) | (yi << 1) | zi];

        unsigned nyi = !yi, nzi = !zi;
        px ^= -(xi & (nyi | zi));
        py ^= -((xi & (yi | zi)) | (yi & nzi));
        pz ^= -((xi & nyi & nzi) | (yi & nzi));

        if (zi)
        {
            unsigned t = px;
            px         = py;
            py         = pz;
            pz         = t;
        }
        else if (!yi)
        {
            unsigned t = px;
            px         = pz;
            pz         = t;
        }
    }
    return key;
}

/* decodeHilbert (sfc/hilbert.hpp:130-173): inverse of the above, least significant octant first */
void cso_decode_hilbert(uint64_t key, int key_bits, unsigned* ixyz)
{
    unsigned px = 0, py = 0, pz = 0;
    for (unsigned level = 0; level < (unsigned)max_level(key_bits); ++level)
    {
        unsigned octant = (unsigned)((key >> (3 * level)) & 7u);
        unsigned xi     = octant >> 2u;
        unsigned yi     = (octant >> 1u) & 1u;
        unsigned zi     = octant & 1u;

        if (yi ^ zi)
        {
            unsigned t = px;
            px         = pz;
            pz         = py;
            py         = t;
        }
        else if ((!xi & !yi & !zi) || (xi & yi & zi))
        {
            unsigned t = px;
            px         = pz;
            pz         = t;
        }

        unsigned mask = (1u << level) - 1u;
        px ^= mask & (-(xi & (yi | zi)));
        py ^= mask & (-((xi & ((!yi) | (!zi))) | ((!xi) & yi & zi)));
        pz ^= mask & (-((xi & (!yi) & (!zi)) | (yi & zi)));

        px |= (xi << level);
        py |= ((xi ^ yi) << level);
        pz |= ((yi ^ zi) << level);
    }
    ixyz[0] = px;
    ixyz[1] = py;
    ixyz[2] = pz;
}

static inline uint64_t isfc(unsigned ix, unsigned iy, unsigned iz, int kind, int key_bits)
{
    return kind == CSO_HILBERT ? cso_ihilbert(ix, iy, iz, key_bits) : cso_imorton(ix, iy, iz, key_bits);
}

/* smallestCommonBox (sfc/common.hpp:342-349) */
static inline void smallest_common_box(uint64_t a, uint64_t b, int key_bits, uint64_t* start, uint64_t* end)
{
    unsigned level = (unsigned)common_prefix(a, b, key_bits) / 3u;
    *start         = enclosing_box_code(a, level, key_bits);
    *end           = *start + node_range(level, key_bits);
}

/* ------------------------------------------------------------------------------------------------------------ */
/* stable sort by key                                                                                            */
/* ------------------------------------------------------------------------------------------------------------ */

typedef struct
{
    uint64_t k;
    uint32_t v;
} kv_pair;

/* Bottom-up merge sort: equal keys keep their input order, which is the contract of std::stable_sort used by
 * sort_by_key (primitives/gather.hpp:42-67). Serial, as in the reference. */
void cso_sort_by_key(uint64_t* keys, uint32_t* values, size_t n)
{
    if (n < 2) return;
    kv_pair* a = (kv_pair*)malloc(n * sizeof(kv_pair));
    kv_pair* b = (kv_pair*)malloc(n * sizeof(kv_pair));
    for (size_t i = 0; i < n; ++i)
    {
        a[i].k = keys[i];
        a[i].v = values[i];
    }
    /* insertion-sort runs of 32 */
    const size_t run = 32;
    for (size_t s = 0; s < n; s += run)
    {
        size_t e = s + run < n ? s + run : n;
        for (size_t i = s + 1; i < e; ++i)
        {
            kv_pair t = a[i];
            size_t j  = i;
            while (j > s && a[j - 1].k > t.k)
            {
                a[j] = a[j - 1];
                --j;
            }
            a[j] = t;
        }
    }
    for (size_t width = run; width < n; width *= 2)
    {
        for (size_t lo = 0; lo < n; lo += 2 * width)
        {
            size_t mid = lo + width < n ? lo + width : n;
            size_t hi  = lo + 2 * width < n ? lo + 2 * width : n;
            size_t i = lo, j = mid, o = lo;
            while (i < mid && j < hi)
                b[o++] = (a[j].k < a[i].k) ? a[j++] : a[i++];
            while (i < mid)
                b[o++] = a[i++];
            while (j < hi)
                b[o++] = a[j++];
        }
        kv_pair* t = a;
        a          = b;
        b          = t;
    }
    for (size_t i = 0; i < n; ++i)
    {
        keys[i]   = a[i].k;
        values[i] = a[i].v;
    }
    free(a);
    free(b);
}

void cso_gather_f64(const uint32_t* perm, const double* in, double* out, size_t n)
{
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < n; ++i)
        out[i] = in[perm[i]];
}

void cso_gather_f32(const uint32_t* perm, const float* in, float* out, size_t n)
{
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < n; ++i)
        out[i] = in[perm[i]];
}

/* ------------------------------------------------------------------------------------------------------------ */
/* cornerstone leaf array                                                                                        */
/* ------------------------------------------------------------------------------------------------------------ */

static inline size_t lower_bound_u64(const uint64_t* a, size_t lo, size_t hi, uint64_t v)
{
    while (lo < hi)
    {
        size_t mid = lo + (hi - lo) / 2;
        if (a[mid] < v)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}
static inline size_t upper_bound_u64(const uint64_t* a, size_t lo, size_t hi, uint64_t v)
{
    while (lo < hi)
    {
        size_t mid = lo + (hi - lo) / 2;
        if (a[mid] <= v)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

/* findSearchBounds (tree/csarray.hpp:100-133): exponential search from a guess index */
void cso_find_search_bounds(int64_t first_idx, uint64_t target, const uint64_t* codes, int64_t n_codes,
                            int key_bits, int64_t* out_lo, int64_t* out_hi)
{
    if (n_codes == 0)
    {
        *out_lo = *out_hi = 0;
        return;
    }
    if (first_idx < 0) first_idx = 0;
    if (first_idx > n_codes - 1) first_idx = n_codes - 1;
    if (target >= node_range(0, key_bits))
    {
        *out_lo = (int64_t)lower_bound_u64(codes, 0, (size_t)n_codes, target);
        *out_hi = n_codes;
        return;
    }
    int64_t d         = (codes[first_idx] < target) ? 1 : -1;
    int64_t t_times_d = (int64_t)target * d;
    int64_t range     = 1;
    int64_t second    = first_idx + d;
    while (0 <= second && second < n_codes && d * (int64_t)codes[second] <= t_times_d)
    {
        range *= 2;
        second = first_idx + range * d;
    }
    if (second < 0) second = 0;
    if (second > n_codes) second = n_codes;
    *out_lo = first_idx < second ? first_idx : second;
    *out_hi = first_idx < second ? second : first_idx;
}

/* computeNodeCounts (tree/csarray.hpp:181-235). Both the plain and the guessed variant return the exact count
 * min(#keys in [tree[i], tree[i+1]), maxCount); the guessed variant narrows the binary search with
 * findSearchBounds around the exclusive scan of the input counts, as updateNodeCount does. */
void cso_node_counts(const uint64_t* tree, uint32_t* counts, int32_t num_nodes, const uint64_t* keys, size_t n,
                     uint32_t max_count, int use_guess, int key_bits)
{
    int32_t first = num_nodes, last = num_nodes;
    if (n > 0)
    {
        first = (int32_t)upper_bound_u64(tree, 0, (size_t)num_nodes, keys[0]) - 1;
        last  = (int32_t)upper_bound_u64(tree, 0, (size_t)num_nodes, keys[n - 1]);
    }
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < first; ++i)
        counts[i] = 0;
#pragma omp parallel for schedule(static)
    for (int32_t i = last; i < num_nodes; ++i)
        counts[i] = 0;

    int32_t nnz           = last - first;
    const uint64_t* ptree = tree + first;
    if (use_guess)
    {
        uint32_t acc = 0;
        for (int32_t i = first; i < first + nnz; ++i)
        {
            uint32_t c = counts[i];
            counts[i]  = acc;
            acc += c;
        }
        /* each guess reads a scanned value that a neighbouring iteration may overwrite; snapshot them first */
        uint32_t* guess = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(num_nodes > 0 ? num_nodes : 1));
        memcpy(guess, counts, sizeof(uint32_t) * (size_t)num_nodes);
#pragma omp parallel for schedule(static)
        for (int32_t i = 0; i < nnz; ++i)
        {
            int32_t sidx = i + first + 1 < num_nodes - 1 ? i + first + 1 : num_nodes - 1;
            int64_t lo, hi;
            cso_find_search_bounds((int64_t)guess[i + first], ptree[i], keys, (int64_t)n, key_bits, &lo, &hi);
            size_t rs = lower_bound_u64(keys, (size_t)lo, (size_t)hi, ptree[i]);
            cso_find_search_bounds((int64_t)guess[sidx], ptree[i + 1], keys, (int64_t)n, key_bits, &lo, &hi);
            size_t re  = lower_bound_u64(keys, (size_t)lo, (size_t)hi, ptree[i + 1]);
            uint32_t c = (uint32_t)(re - rs);
            counts[i + first] = c < max_count ? c : max_count;
        }
        free(guess);
    }
    else
    {
#pragma omp parallel for schedule(static)
        for (int32_t i = 0; i < nnz; ++i)
        {
            size_t rs = lower_bound_u64(keys, 0, n, ptree[i]);
            size_t re = lower_bound_u64(keys, 0, n, ptree[i + 1]);
            size_t c  = re - rs;
            counts[i + first] = (uint32_t)(c < max_count ? c : max_count);
        }
    }
}

/* siblingAndLevel + calculateNodeOp (tree/csarray.hpp:250-290) */
static int node_op(const uint64_t* tree, int32_t i, const uint32_t* counts, unsigned bucket, int key_bits)
{
    uint64_t node  = tree[i];
    unsigned level = tree_level(tree[i + 1] - node, key_bits);
    int sib        = -1;
    if (level > 0)
    {
        sib = (int)octal_digit(node, level, key_bits);
        if (tree[i - sib + 8] != tree[i - sib] + node_range(level - 1, key_bits)) sib = -1;
    }
    if (sib > 0)
    {
        const uint32_t* g = counts + i - sib;
        uint64_t parent   = (uint64_t)g[0] + g[1] + g[2] + g[3] + g[4] + g[5] + g[6] + g[7];
        if (parent <= (uint64_t)bucket) return 0;
    }
    unsigned L = (unsigned)max_level(key_bits);
    uint32_t c = counts[i];
    if (c > bucket * 512u && level + 3 < L) return 4096;
    if (c > bucket * 64u && level + 2 < L) return 512;
    if (c > bucket * 8u && level + 1 < L) return 64;
    if (c > bucket && level < L) return 8;
    return 1;
}

/* rebalanceDecision (tree/csarray.hpp:309-329) */
int cso_rebalance_decision(const uint64_t* tree, const uint32_t* counts, int32_t num_nodes, unsigned bucket,
                           int32_t* ops, int key_bits)
{
    int converged = 1;
#pragma omp parallel for schedule(static) reduction(&& : converged)
    for (int32_t i = 0; i < num_nodes; ++i)
    {
        int op = node_op(tree, i, counts, bucket, key_bits);
        ops[i] = op;
        if (op != 1) converged = 0;
    }
    return converged;
}

/* log8ceil (sfc/common.hpp:108-115) */
static unsigned log8ceil(uint64_t v, int key_bits)
{
    if (v == 0) return 0;
    unsigned lz = (unsigned)clzk(v - 1, key_bits);
    return (unsigned)max_level(key_bits) - (lz - (unsigned)unused_bits(key_bits)) / 3u;
}

/* processNode (tree/csarray.hpp:339-366) */
static void process_node(int32_t i, const uint64_t* tree, const int32_t* ops, uint64_t* nt, int key_bits)
{
    uint64_t node  = tree[i];
    unsigned level = tree_level(tree[i + 1] - node, key_bits);
    int32_t op     = ops[i + 1] - ops[i];
    int32_t out    = ops[i];
    if (op == 1) { nt[out] = node; }
    else if (op == 8)
    {
        for (int s = 0; s < 8; ++s)
            nt[out + s] = node + (uint64_t)s * node_range(level + 1, key_bits);
    }
    else if (op > 8)
    {
        unsigned ld = log8ceil((uint64_t)(unsigned)op, 32);
        for (int s = 0; s < op; ++s)
            nt[out + s] = node + (uint64_t)s * node_range(level + ld, key_bits);
    }
}

/* rebalanceTree (tree/csarray.hpp:375-389): `ops` has num_nodes + 1 entries and is scanned in place */
int32_t cso_rebalance_tree(const uint64_t* tree, int32_t num_nodes, int32_t* ops, uint64_t* new_tree,
                           int32_t new_capacity, int key_bits)
{
    int32_t acc = 0;
    for (int32_t i = 0; i <= num_nodes; ++i)
    {
        int32_t v = (i < num_nodes) ? ops[i] : 0;
        ops[i]    = acc;
        acc += v;
    }
    int32_t nn = ops[num_nodes];
    if (nn > new_capacity) return -nn;
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < num_nodes; ++i)
        process_node(i, tree, ops, new_tree, key_bits);
    new_tree[nn] = tree[num_nodes];
    return nn;
}

/* updateOctree (tree/csarray.hpp:408-426) */
int cso_update_octree(const uint64_t* keys, size_t n, unsigned bucket, uint32_t max_count, uint64_t* tree,
                      uint32_t* counts, int32_t* num_nodes, int32_t capacity, int key_bits)
{
    int32_t L       = *num_nodes;
    int32_t* ops    = (int32_t*)malloc(sizeof(int32_t) * (size_t)(L + 1));
    int converged   = cso_rebalance_decision(tree, counts, L, bucket, ops, key_bits);
    uint64_t* ntree = (uint64_t*)malloc(sizeof(uint64_t) * ((size_t)capacity + 1));
    int32_t nn      = cso_rebalance_tree(tree, L, ops, ntree, capacity, key_bits);
    free(ops);
    if (nn < 0)
    {
        free(ntree);
        *num_nodes = -nn;
        return -1;
    }
    memcpy(tree, ntree, sizeof(uint64_t) * (size_t)(nn + 1));
    free(ntree);
    /* counts.resize keeps the old counts as guesses for the new nodes */
    for (int32_t i = L; i < nn; ++i)
        counts[i] = 0;
    cso_node_counts(tree, counts, nn, keys, n, max_count, 1, key_bits);
    *num_nodes = nn;
    return converged;
}

/* computeOctree (tree/csarray.hpp:429-440) */
int32_t cso_compute_octree(const uint64_t* keys, size_t n, unsigned bucket, uint32_t max_count, uint64_t* tree,
                           uint32_t* counts, int32_t capacity, int key_bits, int* iterations)
{
    int32_t L = 1;
    tree[0]   = 0;
    tree[1]   = node_range(0, key_bits);
    counts[0] = (uint32_t)n;
    int it    = 0;
    for (;;)
    {
        int c = cso_update_octree(keys, n, bucket, max_count, tree, counts, &L, capacity, key_bits);
        ++it;
        if (c < 0) return -L;
        if (c) break;
    }
    if (iterations) *iterations = it;
    return L;
}

/* ------------------------------------------------------------------------------------------------------------ */
/* internal octree                                                                                               */
/* ------------------------------------------------------------------------------------------------------------ */

/* binaryKeyWeight (tree/octree.hpp:55-65) */
int32_t cso_binary_key_weight(uint64_t key, unsigned level, int key_bits)
{
    int32_t ret = 0;
    for (unsigned l = 1; l <= level + 1; ++l)
        ret += digit_weight((int)octal_digit(key, l, key_bits));
    return ret;
}

/* buildOctreeCpu (tree/octree.hpp:167-196) with createUnsortedLayoutCpu (:77-100), getLevelRangeCpu (:151-160)
 * and linkTreeCpu (:114-148) */
void cso_build_octree(const uint64_t* leaves, int32_t L, int key_bits, uint64_t* prefixes, int32_t* child_offsets,
                      int32_t* parents, int32_t* level_range, int32_t* i2l, int32_t* l2i)
{
    int32_t I = (L - 1) / 7;
    int32_t N = L + I;
#pragma omp parallel for schedule(static)
    for (int32_t tid = 0; tid < L; ++tid)
    {
        uint64_t key          = leaves[tid];
        unsigned level        = tree_level(leaves[tid + 1] - key, key_bits);
        prefixes[tid + I]     = encode_placeholder(key, 3 * (int)level, key_bits);
        i2l[tid + I]          = tid + I;
        unsigned prefixLength = (unsigned)common_prefix(key, leaves[tid + 1], key_bits);
        if (prefixLength % 3 == 0 && tid < L - 1)
        {
            int32_t oct   = (tid + cso_binary_key_weight(key, prefixLength / 3, key_bits)) / 7;
            prefixes[oct] = encode_placeholder(key, (int)prefixLength, key_bits);
            i2l[oct]      = oct;
        }
    }
    /* sort_by_key(prefixes, internalToLeaf) */
    uint32_t* vals = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)N);
    for (int32_t i = 0; i < N; ++i)
        vals[i] = (uint32_t)i2l[i];
    cso_sort_by_key(prefixes, vals, (size_t)N);
    for (int32_t i = 0; i < N; ++i)
        i2l[i] = (int32_t)vals[i];
    free(vals);

#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < N; ++i)
        l2i[i2l[i]] = i;
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < N; ++i)
        i2l[i] -= I;

    int maxL = max_level(key_bits);
    for (int level = 0; level <= maxL; ++level)
        level_range[level] =
            (int32_t)lower_bound_u64(prefixes, 0, (size_t)N, encode_placeholder(0, 3 * level, key_bits));
    level_range[maxL + 1] = N;

    memset(child_offsets, 0, sizeof(int32_t) * (size_t)N);
#pragma omp parallel for schedule(static)
    for (int32_t i = 0; i < I; ++i)
    {
        int32_t idxA     = l2i[i];
        uint64_t prefix  = prefixes[idxA];
        uint64_t nodeKey = decode_placeholder(prefix, key_bits);
        unsigned plen    = decode_prefix_length(prefix);
        unsigned level   = plen / 3;
        uint64_t child   = encode_placeholder(nodeKey, (int)plen + 3, key_bits);
        int32_t s        = level_range[level + 1];
        int32_t e        = level_range[level + 2];
        int32_t c        = (int32_t)lower_bound_u64(prefixes, (size_t)s, (size_t)e, child);
        if (c != e && prefixes[c] == child)
        {
            child_offsets[idxA]    = c;
            parents[(c - 1) / 8] = idxA;
        }
    }
}

/* ------------------------------------------------------------------------------------------------------------ */
/* floating-point parts, instantiated for double and float                                                        */
/* ------------------------------------------------------------------------------------------------------------ */

#define REAL double
#define SFX(name) name##_f64
#define RFLOOR floor
#define RRINT rint
#define RSQRT sqrt
#define RABS fabs
#include "cs_oracle_real.inc"
#undef REAL
#undef SFX
#undef RFLOOR
#undef RRINT
#undef RSQRT
#undef RABS

#define REAL float
#define SFX(name) name##_f32
#define RFLOOR floorf
#define RRINT rintf
#define RSQRT sqrtf
#define RABS fabsf
#include "cs_oracle_real.inc"
#undef REAL
#undef SFX
#undef RFLOOR
#undef RRINT
#undef RSQRT
#undef RABS

/* ------------------------------------------------------------------------------------------------------------ */
/* workload generators                                                                                           */
/* ------------------------------------------------------------------------------------------------------------ */

/* Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11). */
static void philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4])
{
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; ++r)
    {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0;
        uint32_t n1 = (uint32_t)p1;
        uint32_t n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        uint32_t n3 = (uint32_t)p0;
        c0 = n0;
        c1 = n1;
        c2 = n2;
        c3 = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

static inline double u01_53(uint32_t a, uint32_t b)
{
    uint64_t m = ((uint64_t)a << 21) ^ (uint64_t)(b >> 11);
    return (double)(m & ((1ull << 53) - 1)) * (1.0 / 9007199254740992.0);
}

/* n doubles uniform in [lo, hi): element i uses counter (i, stream) */
void cso_philox_uniform_f64(uint64_t seed, uint64_t stream, double* out, size_t n, double lo, double hi)
{
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < n; ++i)
    {
        uint32_t ctr[4] = {(uint32_t)i, (uint32_t)(i >> 32), (uint32_t)stream, (uint32_t)(stream >> 32)};
        uint32_t r[4];
        philox4x32_10(ctr, key, r);
        double u = u01_53(r[0], r[1]);
        out[i]   = lo + (hi - lo) * u;
    }
}

/* Plummer sphere with scale radius 1, truncated at rmax: R = (u^(-2/3) - 1)^(-1/2), z = (1 - 2u)R,
 * phi = 2 pi u (the sampling of test/coord_samples/plummer.hpp:15-49, without its 3pi/16 rescale), then shifted to
 * its centre of mass. Particle i draws from counters (i, attempt), so the sample is independent of thread count. */
void cso_plummer_f64(uint64_t seed, double* x, double* y, double* z, size_t n, double rmax)
{
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < n; ++i)
    {
        for (uint32_t attempt = 0;; ++attempt)
        {
            uint32_t ctr[4] = {(uint32_t)i, (uint32_t)(i >> 32), attempt, 0x504c554du};
            uint32_t r[4], s[4];
            philox4x32_10(ctr, key, r);
            ctr[3] = 0x504c554eu;
            philox4x32_10(ctr, key, s);
            double u0 = u01_53(r[0], r[1]);
            double u1 = u01_53(r[2], r[3]);
            double u2 = u01_53(s[0], s[1]);
            if (u0 <= 0.0) continue;
            double R = 1.0 / sqrt(pow(u0, -2.0 / 3.0) - 1.0);
            if (!(R < rmax)) continue;
            double Z     = (1.0 - 2.0 * u1) * R;
            double theta = 2.0 * M_PI * u2;
            double rho   = sqrt(R * R - Z * Z);
            x[i]         = rho * cos(theta);
            y[i]         = rho * sin(theta);
            z[i]         = Z;
            break;
        }
    }
    double cx = 0, cy = 0, cz = 0;
    for (size_t i = 0; i < n; ++i)
    {
        cx += x[i];
        cy += y[i];
        cz += z[i];
    }
    cx /= (double)n;
    cy /= (double)n;
    cz /= (double)n;
#pragma omp parallel for schedule(static)
    for (size_t i = 0; i < n; ++i)
    {
        x[i] -= cx;
        y[i] -= cy;
        z[i] -= cz;
    }
}

int cso_num_threads(void)
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* findNeighbors and computeBoundingBox with double coordinates and float h (Tc = double, Th = float,
 * findneighbors.hpp:77-99, focus/source_center.hpp:28-43): the radii are float expressions, promoted where they meet
 * double distances */
void cso_find_neighbors_f64_hf32(const double* x, const double* y, const double* z, const float* h, uint32_t first,
                                 uint32_t last, const cso_box* box, const int32_t* child_offsets,
                                 const int32_t* parents, const int32_t* internal_to_leaf, const uint32_t* layout,
                                 const double* centers, const double* sizes, float search_ext, unsigned ngmax,
                                 uint32_t* neighbors, uint32_t* counts)
{
    rbox_f64 b  = make_rbox_f64(box);
    int any_pbc = b.pbc[0] || b.pbc[1] || b.pbc[2];
    uint32_t nw = last - first;
#pragma omp parallel for schedule(dynamic, 256)
    for (uint32_t w = 0; w < nw; ++w)
    {
        uint32_t i   = w + first;
        float hi     = h[i];
        float r2     = 4.0f * hi * hi;
        float cellR2 = r2 * search_ext * search_ext;
        counts[w]    = find_neighbors_one_f64(i, x, y, z, (double)r2, (double)cellR2, 2.0 * (double)hi, &b, any_pbc,
                                              child_offsets, parents, internal_to_leaf, layout, centers, sizes, ngmax,
                                              neighbors + (size_t)w * ngmax);
    }
}

void cso_search_boxes_f64_hf32(const double* x, const double* y, const double* z, const float* h,
                               const uint32_t* layout, int32_t first_leaf, int32_t last_leaf, float scale,
                               const int32_t* leaf_to_internal, const double* node_centers, double* search_centers,
                               double* search_sizes)
{
#pragma omp parallel for
    for (int32_t leaf = first_leaf; leaf < last_leaf; ++leaf)
    {
        const double* init = node_centers + 3 * (size_t)leaf_to_internal[leaf];
        double mn[3] = {init[0], init[1], init[2]};
        double mx[3] = {init[0], init[1], init[2]};
        for (uint32_t i = layout[leaf]; i < layout[leaf + 1]; ++i)
        {
            float r     = h[i] * scale;
            double p[3] = {x[i], y[i], z[i]};
            for (int k = 0; k < 3; ++k)
            {
                double a = p[k] - r, c = p[k] + r;
                mn[k]    = a < mn[k] ? a : mn[k];
                mx[k]    = mx[k] < c ? c : mx[k];
            }
        }
        for (int k = 0; k < 3; ++k)
        {
            search_centers[3 * (size_t)leaf + k] = (mx[k] + mn[k]) * 0.5;
            search_sizes[3 * (size_t)leaf + k]   = (mx[k] - mn[k]) * 0.5;
        }
    }
}

#include "cs_oracle_next.inc"

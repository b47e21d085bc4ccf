// Photon KD-tree built on the GPU by parallel median splits.
//
// Same tree as KD_Tree::build_kd_tree (src/KD_Tree.cpp:110-190): an implicit heap
// of 8-byte nodes, root at 1, children 2e and 2e+1.  A node over `count` photons
// splits at the element of rank count/2 along its axis; an odd count keeps that
// median photon in the node (flags 0x90/0xB0/0xF0 | photon index, split = its
// coordinate) and gives count/2 photons to each child; an even count gives the first
// count/2 to the left child and the rest to the right (flags 0x80/0xA0/0xE0, split =
// median coordinate + 1.175494e-38f).  Both children therefore always hold count/2
// photons, so every node on level l holds exactly n >> l photons and the tree shape
// depends only on n.  Leaves (count 1) store the photon index.
//
// The axis is the largest extent of the node's photons computed exactly (the
// reference estimates it from 400 random samples above 500 photons, with a y/z typo
// at src/KD_Tree.cpp:84); the axis choice does not change which photons a radius
// query returns, only the tree's shape.
//
// Alongside the nodes the build leaves the photons in tree order: the photons of the
// subtree at node e occupy one contiguous range [start(e), start(e) + (n >> l)),
// with each odd node's median photon between its children's ranges.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace rc {

struct KdTree {
    long long n = 0;          // photons
    int levels = 0;           // leaf level L = floor(log2 n)
    long long num_nodes = 0;  // node-array length (reference sizing)
    uint2* nodes = nullptr;   // (index word, split bits)
    // photons in tree order (SoA) and their photon-buffer index
    float* x = nullptr; float* y = nullptr; float* z = nullptr;
    uint32_t* id = nullptr;
    // optional node bounding boxes for levels [0, box_levels) (launch_kd_boxes)
    float4* box_lo = nullptr;
    float4* box_hi = nullptr;
    int box_levels = 0;
};

// Start of node e's photon range (root e = 1, level = floor(log2 e)).
__host__ __device__ __forceinline__ long long kd_node_start(long long e, int level, long long n) {
    long long start = 0, c = n;
    for (int b = level - 1; b >= 0; --b) {
        long long half = c >> 1;
        if ((e >> b) & 1) start += half + (c & 1);
        c = half;
    }
    return start;
}

struct KdBuildWork;   // opaque device scratch

// Scratch bytes needed to build over n photons.
size_t kd_scratch_bytes(long long n);

// Build the tree over n photons whose positions are the xyz of pos4[i] (float4).
// All buffers are device memory owned by the caller: tree arrays sized for n (nodes:
// kd_node_array_len(n)), scratch of kd_scratch_bytes(n).  Runs on `stream`.
long long kd_node_array_len(long long n);
// err: device int that receives a non-zero flag if the selection or partition finds
// inconsistent counts (the affected photons are not written).
int kd_build(const float4* pos4, long long n, KdTree& tree, void* scratch, size_t scratch_bytes,
             cudaStream_t stream, int* launches, int* err);

}  // namespace rc

// Multifrontal symbolic analysis (nested dissection) of a symmetric pattern.
#pragma once
#include <cstdint>
#include <vector>

struct NdNode {
    int s = 0;          // DoFs eliminated at this node (front rows 0..s-1)
    int f = 0;          // front size (s + structure)
    int parent = -1;
    int front_off = 0;  // front[front_off .. +f): local DoFs, own first, then structure
    int child_off = 0, nchild = 0;
    int entry_off = 0, nentry = 0;   // original entries assembled here
    int ext_off = 0;    // ext[ext_off .. +(f-s)): this node's structure in the parent's front
    int pad = 0;
    int64_t L_off = 0;  // factor columns: f x s row-major
    int64_t U_off = 0;  // update matrix: (f-s) x (f-s) row-major
};

struct NdSymbolic {
    int n = 0, nnodes = 0, max_f = 0, max_s = 0;
    std::vector<int32_t> perm;      // perm[k] = DoF eliminated k-th
    std::vector<NdNode> node;       // post-order
    std::vector<int32_t> front, child, ent_rel, ent_pos, ext;
    int64_t L_size = 0, U_size = 0;
    // level schedule: nodes grouped by height above the leaves (children
    // always in a lower level), level_nodes[level_ptr[l] .. level_ptr[l+1])
    std::vector<int32_t> level_ptr, level_nodes, level_maxf;
    std::vector<int64_t> uv_off;    // per node: offset of its update vector (f - s values)
    int64_t uv_size = 0;
};

// rowptr/cols: the local pattern (cols local to the problem, diagonal
// included, symmetric); ent_rel is relative to rowptr[0].  Returns 0 on success.
int nd_symbolic_build(int n, const int32_t *rowptr, const int32_t *cols, NdSymbolic *S);

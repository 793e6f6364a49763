// Sparse symmetric LDL^T (multifrontal, supernodal) for the K(2) block that
// the assembly leaves on the device: the GPU counterpart of the reference's
// EquationSolver (EquationSolver.h:19-34; factorizeEquations /
// substituteEquations on a SparseSymMatrix, upper CSR, 1-based).
//
// Symbolic analysis (host, once per pattern): the caller's fill-reducing
// permutation, the elimination tree (Liu), a postorder, column counts from
// the row subtrees, fundamental supernodes merged by a relaxed amalgamation,
// the supernodal row structures, and the maps the device needs: where every
// stored value of the matrix lands in its front, and where every row of a
// child's update matrix lands in its parent's front.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

struct LdltSymbolic {
  int64_t n = 0;
  uint64_t nnz = 0;                 // stored entries of the upper CSR input
  std::vector<int32_t> perm;        // factor order -> input index (0-based)
  // supernodes in postorder: columns [sn_first[s], sn_first[s+1])
  std::vector<int32_t> sn_first;
  std::vector<int64_t> row_ptr;     // rows(s) = rows[row_ptr[s] .. row_ptr[s+1]), sorted,
  std::vector<int32_t> rows;        // the first k(s) are the pivots of s
  std::vector<int32_t> sn_parent;   // -1 at a root
  std::vector<int32_t> child_ptr, child_list;    // children, ascending
  std::vector<int32_t> level;                    // 0 at the leaves
  std::vector<int32_t> level_ptr, level_list;    // supernodes per level
  std::vector<int64_t> rel_ptr;     // per supernode: its update rows' positions in the parent
  std::vector<uint32_t> rel;
  std::vector<uint64_t> front_off;  // m(s)^2 entries per front (column-major)
  std::vector<uint64_t> vec_off;    // m(s) entries per front vector (solve)
  std::vector<uint64_t> a_dest;     // per input slot: index into the front buffer
  // full (both triangles) CSR of the input in input numbering, values by slot (SpMV)
  std::vector<int64_t> full_ptr;
  std::vector<int32_t> full_col;
  std::vector<uint32_t> full_slot;
  // statistics
  uint64_t nnz_L = 0;               // lower-trapezoid entries of all fronts (incl. D)
  double flops = 0.0;               // factorisation flops
  int32_t max_front = 0, max_children = 0;
  int64_t n_sn() const { return (int64_t)sn_first.size() - 1; }
  int32_t m(int64_t s) const { return (int32_t)(row_ptr[s + 1] - row_ptr[s]); }
  int32_t k(int64_t s) const { return sn_first[s + 1] - sn_first[s]; }
};

// iofeir (n+1) / columns: upper CSR, 1-based, sorted per row, diagonal
// present or not; perm (n): a fill-reducing order, perm[new] = input index,
// or null for the identity.  Returns "" or an error message.
// Fill-reducing order for the factorisation without pivoting (order[new] =
// row): geometric nested dissection of the rows' points, then the rows below
// n_dofs that have a stored diagonal, the rows from n_dofs on (MPC / CE
// equations), the rows below n_dofs without a diagonal.
std::string ldlt_nd_order(int64_t n, const uint32_t* iofeir, const uint32_t* columns,
                          const double* points, int64_t n_dofs, int32_t* order);
std::string ldlt_analyze(int64_t n, const uint32_t* iofeir, const uint32_t* columns,
                         const int32_t* perm, LdltSymbolic* out);

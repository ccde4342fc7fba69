// Host-side integer graph work: node adjacency, orderings, colourings and
// the symbolic ILU(k) pattern.  Results are compared bit-for-bit with the
// reference's own arrays.
#pragma once
#include <vector>

namespace a2ds {

// TACSAssembler::computeLocalNodeToNodeCSR (src/TACSAssembler.cpp:1839-1990)
// followed by TacsSortAndUniquifyCSR (src/utils/TacsUtilities.cpp:280): the
// sorted, unique neighbours of every node through the elements, with the
// diagonal unless nodiag.
void node_csr(int nn, int ne, int npe, const int *conn, int nodiag, std::vector<int> &rowp,
              std::vector<int> &cols);

// The reference's approximate-minimum-degree ordering with no interface
// nodes (amd_order_interface, src/bpmat/AMDInterface.cpp), perm[i] = node
// eliminated i-th.  rowp/cols: adjacency without the diagonal (consumed).
int amd_order(int nn, std::vector<int> &rowp, std::vector<int> &cols, std::vector<int> &perm);

// Reverse Cuthill-McKee of a symmetric graph (rowp/cols, diagonal allowed):
// breadth-first level sets from `root` (restarting from the lowest unnumbered
// node for a disconnected graph), neighbours taken in CSR order, numbering
// reversed at the end; passes > 1 restart from the last pass's first node.
// new_vars[old] = new.  Same steps as TacsComputeRCMOrder
// (src/utils/TacsUtilities.cpp:313-426) so the permutation is identical.
int rcm_order(int nn, const std::vector<int> &rowp, const std::vector<int> &cols, int root,
              int passes, std::vector<int> &new_vars);

// Greedy serial multicolouring of a graph: node i takes the smallest colour
// unused by its already-coloured neighbours; new_vars numbers the nodes
// colour by colour, in node order within a colour.  Same steps as
// TacsComputeSerialMultiColor (src/utils/TacsUtilities.cpp:430-490).
// Returns the number of colours.
int multicolor_order(int nn, const std::vector<int> &rowp, const std::vector<int> &cols,
                     std::vector<int> &colors, std::vector<int> &new_vars);

// Greedy element colouring: elements in one colour share no node.
void greedy_element_colors(int nn, int ne, int npe, const int *conn, std::vector<int> &color_ptr,
                           std::vector<int> &color_elems);

// BCSRMat::computeILUk (src/bpmat/BCSRMat.cpp:625-754): the ILU(levFill)
// pattern of a square BCSR pattern (sorted rows with diagonal).  Outputs the
// factor rowp/cols and the diagonal positions.
int ilu_symbolic(int n, const std::vector<int> &rowp, const std::vector<int> &cols, int lev_fill,
                 std::vector<int> &frowp, std::vector<int> &fcols, std::vector<int> &fdiag);

}  // namespace a2ds

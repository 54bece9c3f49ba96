// rs_mech.h -- host-side sparse tables of one mechanism, derived once at rs_create from the
// rs_mechanism arrays (reaction_systems of the .esm file).  Shared by the C-ABI layer, which
// uploads them for the table-walking kernels, and by the specialising code generator.
#pragma once
#include <vector>

namespace rs {

struct MechTables {
  int ns = 0, nr = 0;
  std::vector<int> rptr, rsp, rnu,  // reactant entries (species, stoichiometry) per reaction
      rhs_ptr, rhs_r,               // RHS terms of species s: reactions ascending
      part_r, part_q, part_e,       // partial p = d v_{part_r} / d x_{part_q}
      jac_ptr, jac_slot, jac_diag, jac_part,  // Jacobian entries (row-major) and their terms
      lu_diag,                      // LU slot of pivot k (elimination position)
      ord,                          // species eliminated at position k
      elim_ptr, elim_lik, upd_ptr, upd_dst, upd_src,  // natural-order elimination schedule
      low_ptr, low_row, low_slot,   // forward solve, column k: rows i>k
      up_ptr, up_col, up_slot,      // backward solve, row i: columns j>i (ascending in the
                                    // natural order, descending in the minimum-fill order)
      pupd_ptr, upd_lik,            // per pivot: range of its updates; each update's multiplier
      upc_ptr, upc_row, upc_slot,   // upper factor by columns: column j's rows i<j
      prog_ptr, prog_op,            // rate programs
      slot_row, slot_col;           // (row, col) of each LU slot
  std::vector<double> rhs_c, jac_coef, prog_val, params;
  int nlu = 0, npart = 0, njac = 0, comb = 0;
};

}  // namespace rs

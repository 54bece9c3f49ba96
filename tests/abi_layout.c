/* abi_layout.c -- prints the byte layout of the C ABI's structs (include/reseact_gb300.h) as
 * JSON: for each struct its size and each field's offset.  Built and run by
 * tests/test_abi_layout_cpu.py, which checks the Python ctypes mirrors and the Julia isbits
 * mirrors against it; its output at the header's current layout is committed as
 * tests/golden/abi_layout.json. */
#include <stddef.h>
#include <stdio.h>

#include "reseact_gb300.h"

static int first_struct = 1, first_field = 1;
static void begin(const char* name, size_t size) {
  printf("%s\n  \"%s\": {\"size\": %zu, \"fields\": {", first_struct ? "{" : ",", name, size);
  first_struct = 0;
  first_field = 1;
}
static void field(const char* name, size_t off) {
  printf("%s\"%s\": %zu", first_field ? "" : ", ", name, off);
  first_field = 0;
}
static void end(void) { printf("}}"); }
#define F(T, m) field(#m, offsetof(T, m))

int main(void) {
  begin("rs_mechanism", sizeof(rs_mechanism));
  F(rs_mechanism, n_species); F(rs_mechanism, n_reactions); F(rs_mechanism, n_params);
  F(rs_mechanism, combinatoric); F(rs_mechanism, react_ptr); F(rs_mechanism, react_species);
  F(rs_mechanism, react_nu); F(rs_mechanism, prod_ptr); F(rs_mechanism, prod_species);
  F(rs_mechanism, prod_coef); F(rs_mechanism, prog_ptr); F(rs_mechanism, prog_op);
  F(rs_mechanism, prog_val); F(rs_mechanism, params);
  end();
  begin("rs_grid", sizeof(rs_grid));
  F(rs_grid, nlon); F(rs_grid, nlat); F(rs_grid, nlev); F(rs_grid, lon_bc); F(rs_grid, lat_bc);
  F(rs_grid, lon0_deg); F(rs_grid, dlon_deg); F(rs_grid, lat0_deg); F(rs_grid, dlat_deg);
  end();
  begin("rs_controller", sizeof(rs_controller));
  F(rs_controller, beta1); F(rs_controller, beta2); F(rs_controller, qmin);
  F(rs_controller, qmax); F(rs_controller, gamma); F(rs_controller, qsteady_min);
  F(rs_controller, qsteady_max); F(rs_controller, qoldinit);
  end();
  begin("rs_config", sizeof(rs_config));
  F(rs_config, api_version); F(rs_config, device); F(rs_config, grid);
  F(rs_config, has_air_mass); F(rs_config, do_transport); F(rs_config, do_chemistry);
  F(rs_config, mech); F(rs_config, rtol_T); F(rs_config, atol_T); F(rs_config, rtol_C);
  F(rs_config, atol_C); F(rs_config, ctrl_T); F(rs_config, ctrl_C); F(rs_config, maxiters);
  F(rs_config, clamp_nonneg); F(rs_config, precision); F(rs_config, chem_mode);
  end();
  begin("rs_forcing", sizeof(rs_forcing));
  F(rs_forcing, mx); F(rs_forcing, my); F(rs_forcing, mz); F(rs_forcing, flux_omega);
  F(rs_forcing, dp); F(rs_forcing, qbc_w); F(rs_forcing, qbc_e); F(rs_forcing, qbc_s);
  F(rs_forcing, qbc_n); F(rs_forcing, temperature); F(rs_forcing, pressure);
  F(rs_forcing, emission); F(rs_forcing, pblh); F(rs_forcing, ps); F(rs_forcing, hyb_a);
  F(rs_forcing, hyb_b); F(rs_forcing, tau_pblmix); F(rs_forcing, dps_dt);
  end();
  begin("rs_stats", sizeof(rs_stats));
  F(rs_stats, naT); F(rs_stats, nrT); F(rs_stats, naC); F(rs_stats, nrC); F(rs_stats, dtT_end);
  F(rs_stats, dtC_end); F(rs_stats, tT_end); F(rs_stats, tC_end); F(rs_stats, chem_cell_steps);
  F(rs_stats, kernel_launches); F(rs_stats, status);
  end();
  begin("rs_solve_opts", sizeof(rs_solve_opts));
  F(rs_solve_opts, macro_dt); F(rs_solve_opts, min_macro_dt); F(rs_solve_opts, forcing_tstops);
  F(rs_solve_opts, n_tstops); F(rs_solve_opts, refresh); F(rs_solve_opts, on_bisect);
  F(rs_solve_opts, user);
  end();
  begin("rs_solve_result", sizeof(rs_solve_result));
  F(rs_solve_result, naT); F(rs_solve_result, nrT); F(rs_solve_result, naC);
  F(rs_solve_result, nrC); F(rs_solve_result, nmacro); F(rs_solve_result, nbisect);
  F(rs_solve_result, nrefresh); F(rs_solve_result, status); F(rs_solve_result, pad);
  end();
  printf("\n}\n");
  return 0;
}

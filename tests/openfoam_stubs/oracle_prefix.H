// Points the shim's C-ABI calls at the oracle library, which exports the
// same functions under the icsref_ prefix (CPU runs of the shim test).
#pragma once
#define ics_default_config icsref_default_config
#define ics_create icsref_create
#define ics_destroy icsref_destroy
#define ics_set_config icsref_set_config
#define ics_last_error icsref_last_error
#define ics_set_conservative icsref_set_conservative
#define ics_set_boundary_state icsref_set_boundary_state
#define ics_calc_flux icsref_calc_flux
#define ics_residual icsref_residual
#define ics_assemble_jacobian icsref_assemble_jacobian
#define ics_solve_increment icsref_solve_increment

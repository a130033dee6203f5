// options.hpp -- process-wide launch options (see accspmm_set_option).
#pragma once

namespace accspmm {

// Current value of an ACCSPMM_OPT_* option (environment read once, then
// accspmm_set_option).
int option(int id);
int set_option(int id, int value);
// A knob of the measurement build's variant kernels (ACCSPMM_NW, _HINTS,
// _ORDER, _MINB, _U, _STAGE_V ...), read from the environment once per name.
int lab_env(const char* name, int dflt);

}  // namespace accspmm

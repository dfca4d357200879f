/* Configuration header normally generated by the reference's CMake step
 * (src/meraxes_conf.h.in); values are the CMake defaults. */
#define N_HISTORY_SNAPS 17
#define MERAXES_GITREF_STR "oracle"
#define MERAXES_GITDIFF_STR ""
#define FEATURE_FLAG_CALC_MAGS 0

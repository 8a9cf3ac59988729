// Persistent single-graph peel kernel (and, built with KC_CHECKED, its
// bounds-checked twin); the device code is in kc_peel_impl.cuh.
#include "kc_peel_impl.cuh"

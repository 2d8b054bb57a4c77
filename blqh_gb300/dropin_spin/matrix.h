// Drop-in matrix.h for the spinful model: the host containers Vec / Mat are the
// same as the spinless drop-in's (BLQH_with_spin/matrix.h declares the same
// classes as BLQH_without_spin/matrix.h).
#include "../dropin/matrix.h"

// Drop-in matrix.h for the monolayer: the host containers Vec / Mat are the
// spinless drop-in's (Monolayer/matrix.h declares the same classes as
// BLQH_without_spin/matrix.h).
#include "../dropin/matrix.h"

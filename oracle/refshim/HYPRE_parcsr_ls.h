/* HYPRE stand-in header (test infrastructure): everything is declared in HYPRE.h. */
#include "HYPRE.h"

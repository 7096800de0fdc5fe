/* Minimal stand-in for dohp.h (oracle/_ref build only; test infrastructure). */
#include <math.h>
#include <stdio.h>
#include "dohptype.h"
#define dPragmaGCC(a)

/* Minimal stand-in for dohp's type header so that the reference's own polylib.c and
 * inlinetmulthex.h compile without PETSc (oracle/_ref build only; test infrastructure). */
#ifndef ORACLE_REF_SHIM_DOHPTYPE_H
#define ORACLE_REF_SHIM_DOHPTYPE_H
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
typedef int dInt;
typedef double dReal;
typedef double dScalar;
typedef int dErr;
typedef enum { NOT_SET_VALUES, INSERT_VALUES, ADD_VALUES } InsertMode;
#define dFunctionBegin
#define dFunctionReturn(x) return (x)
#define dCHK(e) do { if (e) return (e); } while (0)
#define dERROR(comm, code, ...) return (code)
#define dMemzero(p, n) (memset((p), 0, (n)), 0)
#define PetscLogFlops(x) 0
#define PETSC_COMM_SELF 0
#endif

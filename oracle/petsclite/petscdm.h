/* petsclite: everything lives in petsc.h */
#include "petsc.h"

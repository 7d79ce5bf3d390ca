/*
 * nosh_solver.c -- CPU FP64 Newton / preconditioned-MINRES restatement.
 *
 * TEST INFRASTRUCTURE ONLY (parity checker for the unpinned solver parts and
 * the timed CPU baseline).  Filled in together with the solver it checks.
 */
#include "nosh_oracle.h"

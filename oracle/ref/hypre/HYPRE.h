/*
 * Stand-in for the one HYPRE name that src/methods/solvers/MatrixSolver.h uses
 * (HYPRE_Int). Test infrastructure only: the harness in ../ref_implicit.cpp
 * compiles the reference's FVM_TVD_IMPLICIT without HYPRE, whose sources are not
 * part of the reference tree, and supplies the matrix solver itself.
 */
#ifndef ORACLE_STUB_HYPRE_H
#define ORACLE_STUB_HYPRE_H
typedef int HYPRE_Int;
#endif

// Set-up calls of the MPI / Kokkos stand-ins, made by ref_harness.cpp.
#pragma once

// Number of ranks (threads) of the run and OpenMP threads per rank (0: the
// OpenMP default divided among the ranks).  Call before starting ranks.
void imexref_set_world(int size, int threads);
// Rank of the calling thread.
void imexref_set_rank(int rank);
int imexref_threads();

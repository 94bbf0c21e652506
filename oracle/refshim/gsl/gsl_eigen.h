/* Empty stand-in: basis_optimisation_mpi.c includes it but calls nothing from it. */

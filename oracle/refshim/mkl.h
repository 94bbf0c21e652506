/* Empty stand-in for <mkl.h>: tetrapyd_tools.c includes it but calls nothing from it. */

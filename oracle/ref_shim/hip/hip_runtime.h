/* Empty stand-in for the HIP runtime header: the reference's host wrappers
 * include it unconditionally, but its CPU (OpenMP) build uses nothing from it. */

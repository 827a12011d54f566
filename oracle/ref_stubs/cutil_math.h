/* Stand-in for the CUDA 4 SDK math helper header the reference includes; its
   GPU kernels use nothing from it (test infrastructure). */

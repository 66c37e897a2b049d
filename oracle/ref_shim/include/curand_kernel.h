/* Empty stand-in: the CUDA declarations the reference needs come from ref_shim.h. */

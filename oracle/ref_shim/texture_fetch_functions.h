/* Empty stand-in: tex1Dfetch for the reference's texture references is
 * defined in the shim cuda_texture_types.h of this directory. */

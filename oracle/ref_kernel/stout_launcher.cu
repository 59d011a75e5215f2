// Launcher of the reference's CUDA stout-smearing kernel (test infrastructure).
//
// lattice/generator/stout_smear.cu:159-245 defines the kernel as a template
// that CuPy instantiates by name at run time.  Here the file is included
// unmodified from the reference source tree (path given by -DED_REF_STOUT_CU)
// with __global__ read as __device__, and one extern "C" kernel calls its
// double instantiation, so every thread runs the reference's own body with
// the reference's launch geometry: grid (Lx*Ly*Lz, 3), block (Lt)
// (lattice/generator/eigenvector.py:197-199).
#pragma push_macro("__global__")
#undef __global__
#define __global__ __device__
#include ED_REF_STOUT_CU
#pragma pop_macro("__global__")

extern "C" __global__ void ed_ref_stout_smear_f64(complex<double>* U_out, const complex<double>* U_in, double rho,
                                                  int Lx, int Ly, int Lz, int Lt) {
  stout_smear<double>(U_out, U_in, rho, Lx, Ly, Lz, Lt);
}

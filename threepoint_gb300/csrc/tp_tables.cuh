#pragma once
#include "tp_bispec.cuh"
#include "tp_internal.cuh"

namespace tp {

// Uploads the Gauss-Legendre abscissae/weights of the 96-node line-of-sight
// rules (constant memory of tp_tables.cu) to the current device.
void upload_gauss_nodes();

// Launches the table build for n cosmologies on stream s: norm, f_K, g, D1,
// r_sigma, n_eff, ncur, then the per-node coefficient blocks (NC_* FP64 and
// FP32 rows, NF_* FP32 rows of the point path, Halofit rows). d_eh must hold
// make_eh_const(c, 1.0) on entry; its ehc is rescaled by norm^2 on exit.
cudaError_t build_tables(const CosmoDev* d_cos, EHConst* d_eh, const double* d_nz, int nz_stride, TablesDev* d_tab,
                         double* d_ncoef, float* d_ncoef_f, float* d_fcoef_f, double* d_hcoef, float* d_hcoef_f,
                         double* d_wscale64,
                         double* d_wscale32, CosmoK<double>* d_ck64, CosmoK<float>* d_ck32, float4* d_plt,
                         double* d_ehg, int n, cudaStream_t s);

// Fills the node rows (HN_*) of the halo-model tables of cosmology ci on
// stream s from its z-tables (launches one small kernel).
cudaError_t build_halo_nodes(const CosmoDev* d_cos, const TablesDev* d_tab, int ci, HaloTab* d_halo, cudaStream_t s);

}  // namespace tp

/*
 * mceliece.h -- the part of libmceliece's public C API (doc/api.md of
 * libmceliece-20250507: keypair returns void, enc/dec return int) that the
 * reference's GPU benchmark harness calls, for the five base sets.
 *
 * TEST INFRASTRUCTURE ONLY: lets oracle/build_ref_gpu.py compile that
 * harness against oracle/_ref/libmcref.so (the same libmceliece `vec` code)
 * instead of an installed libmceliece. The engine never includes it.
 */
#ifndef GMC_REF_GPU_MCELIECE_H
#define GMC_REF_GPU_MCELIECE_H

#ifdef __cplusplus
extern "C" {
#endif

#define GMC_REF_GPU_DECLARE(set)                                                         \
  void mceliece_kem_##set##_keypair(unsigned char *pk, unsigned char *sk);               \
  int mceliece_kem_##set##_enc(unsigned char *c, unsigned char *k, const unsigned char *pk); \
  int mceliece_kem_##set##_dec(unsigned char *k, const unsigned char *c, const unsigned char *sk);

GMC_REF_GPU_DECLARE(348864)
GMC_REF_GPU_DECLARE(460896)
GMC_REF_GPU_DECLARE(6688128)
GMC_REF_GPU_DECLARE(6960119)
GMC_REF_GPU_DECLARE(8192128)

#undef GMC_REF_GPU_DECLARE

#ifdef __cplusplus
}
#endif
#endif

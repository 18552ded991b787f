/* Stand-in for libmceliece's generated crypto_sort_int32.h: the int32 sort
 * is compiled once (portable4) under the name mcref_sort_int32. */
#ifndef crypto_sort_int32_h
#define crypto_sort_int32_h
#define crypto_sort_int32 mcref_sort_int32
extern void crypto_sort_int32(void *, long long);
#endif

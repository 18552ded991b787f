/* Stand-in for libmceliece's generated crypto_sort_int64.h: the int64 sort
 * is compiled once (portable4) under the name mcref_sort_int64. */
#ifndef crypto_sort_int64_h
#define crypto_sort_int64_h
#define crypto_sort_int64 mcref_sort_int64
extern void crypto_sort_int64(void *, long long);
#endif

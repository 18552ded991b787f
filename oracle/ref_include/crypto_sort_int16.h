/* Stand-in for libmceliece's generated crypto_sort_int16.h: the int16 sort
 * is compiled once (portable4) under the name mcref_sort_int16. */
#ifndef crypto_sort_int16_h
#define crypto_sort_int16_h
#define crypto_sort_int16 mcref_sort_int16
extern void crypto_sort_int16(void *, long long);
#endif

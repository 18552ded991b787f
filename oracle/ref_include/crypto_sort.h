/* Stand-in for libmceliece's generated crypto_sort.h, seen by the sort
 * sources themselves; crypto_sort is renamed per sort on the command line. */
#ifndef crypto_sort_h
#define crypto_sort_h
extern void crypto_sort(void *, long long);
#endif

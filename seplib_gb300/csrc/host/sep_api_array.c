/*
 * sep_api_array.c - zero-filled host arrays of the sep C API (reference
 * source/separray.c): vectors, row-pointer matrices and tensors, their
 * release and fills.
 */
#include <stdlib.h>
#include "sep.h"
#include "separray.h"

static void *zalloc(size_t n, size_t size, const char *who)
{
	void *p = calloc(n ? n : 1, size);
	if (!p) sep_error("%s: Couldn't allocate memory", who);
	return p;
}

double *sep_vector(size_t length) { return zalloc(length, sizeof(double), __func__); }
int *sep_vector_int(size_t length) { return zalloc(length, sizeof(int), __func__); }

#define ROWS(T, name)                                                           \
	T **name(size_t nrow, size_t ncol)                                      \
	{                                                                       \
		T **m = zalloc(nrow, sizeof(T *), __func__);                    \
		for (size_t i = 0; i < nrow; i++) m[i] = zalloc(ncol, sizeof(T), __func__); \
		return m;                                                       \
	}
ROWS(double, sep_matrix)
ROWS(int, sep_matrix_int)
ROWS(float, sep_matrix_float)

#define SLABS(T, name, rows)                                                    \
	T ***name(size_t n1, size_t n2, size_t n3)                              \
	{                                                                       \
		T ***t = zalloc(n1, sizeof(T **), __func__);                    \
		for (size_t i = 0; i < n1; i++) t[i] = rows(n2, n3);            \
		return t;                                                       \
	}
SLABS(double, sep_tensor, sep_matrix)
SLABS(int, sep_tensor_int, sep_matrix_int)
SLABS(float, sep_tensor_float, sep_matrix_float)

#define FREE_ROWS(T, name)                                                      \
	void name(T **m, size_t nrow)                                           \
	{                                                                       \
		if (!m) return;                                                 \
		for (size_t i = 0; i < nrow; i++) free(m[i]);                   \
		free(m);                                                        \
	}
FREE_ROWS(double, sep_free_matrix)
FREE_ROWS(int, sep_free_matrix_int)
FREE_ROWS(float, sep_free_matrix_float)

#define FREE_SLABS(T, name, rows)                                               \
	void name(T ***t, size_t n1, size_t n2)                                 \
	{                                                                       \
		if (!t) return;                                                 \
		for (size_t i = 0; i < n1; i++) rows(t[i], n2);                 \
		free(t);                                                        \
	}
FREE_SLABS(double, sep_free_tensor, sep_free_matrix)
FREE_SLABS(int, sep_free_tensor_int, sep_free_matrix_int)
FREE_SLABS(float, sep_free_tensor_float, sep_free_matrix_float)

void sep_vector_set(double *a, size_t length, double value)
{
	for (size_t i = 0; i < length; i++) a[i] = value;
}

void sep_vector_int_set(int *a, size_t length, int value)
{
	for (size_t i = 0; i < length; i++) a[i] = value;
}

void sep_matrix_set(double **a, size_t nrow, size_t ncol, double value)
{
	for (size_t i = 0; i < nrow; i++) sep_vector_set(a[i], ncol, value);
}

void sep_matrix_int_set(int **a, size_t nrow, size_t ncol, int value)
{
	for (size_t i = 0; i < nrow; i++) sep_vector_int_set(a[i], ncol, value);
}

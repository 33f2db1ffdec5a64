/*
 * separray.h - zero-filled host arrays (reference include/separray.h:30-306,
 * the allocation, fill and release helpers).  Allocation failures end the
 * program with sep_error, as in the reference.  Matrices and tensors are
 * arrays of row pointers.
 */
#ifndef SEP_GB300_SEPARRAY_H
#define SEP_GB300_SEPARRAY_H

#include <stddef.h>

double *sep_vector(size_t length);
double **sep_matrix(size_t nrow, size_t ncol);
double ***sep_tensor(size_t n1, size_t n2, size_t n3);
int *sep_vector_int(size_t length);
int **sep_matrix_int(size_t nrow, size_t ncol);
int ***sep_tensor_int(size_t n1, size_t n2, size_t n3);
float **sep_matrix_float(size_t nrow, size_t ncol);
float ***sep_tensor_float(size_t n1, size_t n2, size_t n3);

void sep_free_matrix(double **ptr, size_t nrow);
void sep_free_tensor(double ***a, size_t n1, size_t n2);
void sep_free_matrix_int(int **ptr, size_t nrow);
void sep_free_tensor_int(int ***ptr, size_t n1, size_t n2);
void sep_free_matrix_float(float **ptr, size_t nrow);
void sep_free_tensor_float(float ***a, size_t n1, size_t n2);

void sep_vector_set(double *a, size_t length, double value);
void sep_matrix_set(double **a, size_t nrow, size_t ncol, double value);
void sep_vector_int_set(int *a, size_t length, int value);
void sep_matrix_int_set(int **a, size_t nrow, size_t ncol, int value);

#endif

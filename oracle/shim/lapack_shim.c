/* LAPACK entry points the reference calls (dsyevd_, zheevd_), forwarded to the
 * LP64 LAPACK that scipy ships inside its bundled OpenBLAS, whose symbols carry
 * a scipy_ prefix. Used only by the out-of-tree reference build in oracle/_ref. */
typedef struct { double re, im; } zcplx;
extern int scipy_dsyevd_(char*, char*, int*, double*, int*, double*, double*, int*, int*, int*, int*);
extern int scipy_zheevd_(char*, char*, int*, zcplx*, int*, double*, zcplx*, int*, double*, int*, int*, int*, int*);
int dsyevd_(char* jobz, char* uplo, int* n, double* a, int* lda, double* w, double* work, int* lwork, int* iwork,
            int* liwork, int* info) {
  return scipy_dsyevd_(jobz, uplo, n, a, lda, w, work, lwork, iwork, liwork, info);
}
int zheevd_(char* jobz, char* uplo, int* n, zcplx* a, int* lda, double* w, zcplx* work, int* lwork, double* rwork,
            int* lrwork, int* iwork, int* liwork, int* info) {
  return scipy_zheevd_(jobz, uplo, n, a, lda, w, work, lwork, rwork, lrwork, iwork, liwork, info);
}

# Sourced by the block2 build recipes.  block2 declares its BLAS/LAPACK calls
# as Fortran symbols (dgemm_, dsyev_, ...; src/core/matrix_functions.hpp:37-280).
# The BLAS used here is the LP64 OpenBLAS that scipy bundles, whose symbols
# carry a scipy_ prefix; these -D flags rename block2's declarations to it.
# Sets: B2G_BLAS (library path), B2G_BLAS_DEFS (compiler flags).
B2G_BLAS_DIR="$(python3 -c 'import scipy, os; print(os.path.join(os.path.dirname(scipy.__file__), os.pardir, "scipy.libs"))')"
B2G_BLAS="$(ls "$B2G_BLAS_DIR"/libscipy_openblas*.so | head -1)"
B2G_BLAS_DEFS="-D_F77UNDERSCORE"
for s in caxpy ccopy cdotc cgeev cgelqf cgels cgemm cgemv cgeqp3 cgeqrf cgesv cgesvd cgetrf cgetri cheev chegv clacpy cscal csscal cunglq cungqr \
         daxpy dcopy ddot dgeev dgelqf dgels dgemm dgemv dgeqp3 dgeqrf dgesv dgesvd dgetrf dgetri dlacpy dnrm2 dorglq dorgqr dscal dsyev dsygv dznrm2 \
         saxpy scnrm2 scopy sdot sgeev sgegv sgelqf sgels sgemm sgemv sgeqp3 sgeqrf sgesv sgesvd sgetrf sgetri slacpy snrm2 sorglq sorgqr sscal ssyev ssygv \
         zaxpy zcopy zdotc zdscal zgeev zgelqf zgels zgemm zgemv zgeqp3 zgeqrf zgesv zgesvd zgetrf zgetri zheev zhegv zlacpy zscal zunglq zungqr; do
  B2G_BLAS_DEFS="$B2G_BLAS_DEFS -D${s}_=scipy_${s}_"
done

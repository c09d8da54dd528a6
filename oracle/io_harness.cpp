// Test-infrastructure harness (ORACLE, never the product) around two more of
// the reference's unmodified CPU sources:
//
//   IOfn.cpp    read_G_sparse   the COO text reader (IOfn.cpp:21-54)
//   Pvalue.cpp  Calculate_Pvalue and helpers: correlation, t statistic and
//               the incomplete-beta p-value (Pvalue.cpp:85-235)
//
// usage: io_harness readcoo FILE N1 N2 DATATYPE
//        io_harness timecoo FILE N1 N2 DATATYPE  -> "seconds nnz" of one read
//          -> "n1 n2 nnz" then "row col value" (0-based, %.17g) of the
//             reader's Eigen matrix, column by column
//        io_harness pvalue FILE LEN
//          -> FILE holds 2*LEN numbers (x then y); prints
//             "correlation tstat pvalue" (%.17g)

#include "stdafx.h"

using namespace Eigen;
using namespace std;

int NX, NA, NB, NC, KHID, DATATYPE;
double alpha0;
const char* FILE_Gb_a = 0;
const char* FILE_Gc_a = 0;

int main(int argc, char** argv) {
  if (argc >= 6 && string(argv[1]) == "readcoo") {
    DATATYPE = atoi(argv[5]);
    SparseMatrix<double> m = read_G_sparse(argv[2], (char*)"G", atoi(argv[3]), atoi(argv[4]));
    fprintf(stdout, "%ld %ld %ld\n", (long)m.rows(), (long)m.cols(), (long)m.nonZeros());
    for (int k = 0; k < m.outerSize(); ++k)
      for (SparseMatrix<double>::InnerIterator it(m, k); it; ++it)
        fprintf(stdout, "%ld %ld %.17g\n", (long)it.row(), (long)it.col(), it.value());
    return 0;
  }
  if (argc >= 6 && string(argv[1]) == "timecoo") {  // seconds of one read_G_sparse call
    DATATYPE = atoi(argv[5]);
    clock_t t0 = clock();
    SparseMatrix<double> m = read_G_sparse(argv[2], (char*)"G", atoi(argv[3]), atoi(argv[4]));
    fprintf(stdout, "%.6f %ld\n", (double)(clock() - t0) / CLOCKS_PER_SEC, (long)m.nonZeros());
    return 0;
  }
  if (argc >= 4 && string(argv[1]) == "pvalue") {
    const long len = atol(argv[3]);
    vector<double> x(len), y(len);
    FILE* f = fopen(argv[2], "r");
    if (!f) return 1;
    for (long i = 0; i < len; ++i)
      if (fscanf(f, "%lf", &x[i]) != 1) return 1;
    for (long i = 0; i < len; ++i)
      if (fscanf(f, "%lf", &y[i]) != 1) return 1;
    fclose(f);
    const double r = Calculate_Correlation(x.data(), y.data(), len);
    const double t = Calculate_Tstat(x.data(), y.data(), len);
    const double p = Calculate_Pvalue(x.data(), y.data(), len);
    fprintf(stdout, "%.17g %.17g %.17g\n", r, t, p);
    return 0;
  }
  fprintf(stderr, "usage: %s readcoo FILE N1 N2 DATATYPE | pvalue FILE LEN\n", argv[0]);
  return 2;
}

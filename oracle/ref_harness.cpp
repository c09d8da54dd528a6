// Test-infrastructure harness around the reference's own CPU implementation.
//
// This file is part of the ORACLE (test infrastructure), never of the product.  It links
// the unmodified reference sources CommunityDetectionSoftware_CPU/CommunityDetection/
// {IOfn,Probability,Spectral,Util}.cpp (vendored Eigen 3.2.1) and replaces only
// the reference's `main` (CommunityDetection.cpp:16-149) so that every stage's
// output can be dumped at full precision (%.17g) for the golden fixtures:
//
//   stage                      reference call site
//   -------------------------  --------------------------------------------
//   whitening                  second_whiten           Util.cpp:38-127
//   sketches R_c, R_b, R_a     random_embedding_mat    Spectral.cpp:118-134
//   whitened data / means      CommunityDetection.cpp:66-68
//   batch tensor power (STPM)  tensorDecom_alpha0      Util.cpp:131-184
//   unwhitening                CommunityDetection.cpp:98-108
//   concat + normalisation     CommunityDetection.cpp:118-139, Probability.cpp:89-121
//   per-sample SGD step        Diff_Loss               Util.cpp:257-284
//   writers                    write_pi                IOfn.cpp:57-67
//
// Determinism: the reference seeds with srand(clock()) (Spectral.cpp:120,138);
// the recipe links with -Wl,--wrap=srand and srand_shim.c forces a fixed seed,
// so every random_embedding_mat call restarts the same rand() stream.  The
// initial Phi0 of tensorDecom_alpha0 (Util.cpp:134-142) is MatrixXd::Random
// drawn from the rand() state left by the last sketch (R_a, 2*NA draws); the
// harness reproduces that state to export Phi0.
//
// Input graphs are read from 1-based COO text ("row col" per line, the
// reference's file contract) by this harness's own parser, which does not
// repeat the reference reader's final-line duplication (IOfn.cpp:36-49).
//
// usage: ref_harness IN_DIR OUT_DIR NX NA NB NC KHID ALPHA0

#include "stdafx.h"
#include <sys/stat.h>
#include <chrono>

using namespace Eigen;
using namespace std;

int NX, NA, NB, NC, KHID, DATATYPE;
double alpha0;
const char* FILE_Gb_a = 0;
const char* FILE_Gc_a = 0;

static SparseMatrix<double> load_coo(const string& path, int n1, int n2) {
  FILE* f = fopen(path.c_str(), "r");
  if (!f) { fprintf(stderr, "cannot open %s\n", path.c_str()); exit(1); }
  vector<Triplet<double> > t;
  long r, c;
  while (fscanf(f, "%ld %ld", &r, &c) == 2) {
    if (r < 1 || r > n1 || c < 1 || c > n2) { fprintf(stderr, "bad index in %s\n", path.c_str()); exit(1); }
    t.push_back(Triplet<double>((int)r - 1, (int)c - 1, 1.0));
  }
  fclose(f);
  SparseMatrix<double> m(n1, n2);
  m.setFromTriplets(t.begin(), t.end());
  m.makeCompressed();
  return m;
}

static void dump(const string& path, const MatrixXd& m) {
  FILE* f = fopen(path.c_str(), "w");
  if (!f) { fprintf(stderr, "cannot write %s\n", path.c_str()); exit(1); }
  fprintf(f, "%ld %ld\n", (long)m.rows(), (long)m.cols());
  for (long i = 0; i < m.rows(); ++i) {
    for (long j = 0; j < m.cols(); ++j) fprintf(f, j ? " %.17g" : "%.17g", m(i, j));
    fprintf(f, "\n");
  }
  fclose(f);
}

static double now_s() {
  return chrono::duration<double>(chrono::steady_clock::now().time_since_epoch()).count();
}

int main(int argc, char** argv) {
  if (argc < 9) {
    fprintf(stderr, "usage: %s IN_DIR OUT_DIR NX NA NB NC KHID ALPHA0\n", argv[0]);
    return 2;
  }
  string in = argv[1], out = argv[2];
  NX = atoi(argv[3]); NA = atoi(argv[4]); NB = atoi(argv[5]); NC = atoi(argv[6]);
  KHID = atoi(argv[7]); alpha0 = atof(argv[8]); DATATYPE = 0;
  mkdir(out.c_str(), 0755);
  FILE* tf = fopen((out + "/timing.txt").c_str(), "w");

  double t0 = now_s();
  SparseMatrix<double> Gx_a = load_coo(in + "/Gx_a.txt", NX, NA);
  SparseMatrix<double> Gx_b = load_coo(in + "/Gx_b.txt", NX, NB);
  SparseMatrix<double> Gx_c = load_coo(in + "/Gx_c.txt", NX, NC);
  SparseMatrix<double> Gb_a = load_coo(in + "/Gb_a.txt", NB, NA);
  SparseMatrix<double> Gc_a = load_coo(in + "/Gc_a.txt", NC, NA);
  double t1 = now_s();
  fprintf(tf, "read %.6f\n", t1 - t0);

  // whitening (CommunityDetection.cpp:58-68)
  SparseMatrix<double> W(NA, KHID), Zb1(NA, KHID), Zb2(KHID, NB), Zc1(NA, KHID), Zc2(KHID, NC);
  VectorXd mu_a(NA), mu_b(NB), mu_c(NC);
  second_whiten(Gx_a, Gx_b, Gx_c, W, Zb1, Zb2, Zc1, Zc2, mu_a, mu_b, mu_c);
  SparseMatrix<double> Da = W.transpose() * Gx_a.transpose();
  VectorXd Da_mu = W.transpose() * mu_a;
  SparseMatrix<double> Db = (W.transpose() * Zb1) * Zb2 * Gx_b.transpose();
  VectorXd Db_mu = (W.transpose() * Zb1) * Zb2 * mu_b;
  SparseMatrix<double> Dc = (W.transpose() * Zc1) * Zc2 * Gx_c.transpose();
  VectorXd Dc_mu = (W.transpose() * Zc1) * Zc2 * mu_c;
  double t2 = now_s();
  fprintf(tf, "whiten %.6f\n", t2 - t1);

  // the three sketches exactly as second_whiten drew them (same seeded stream)
  MatrixXd Rc = MatrixXd(random_embedding_mat(NB, 2 * KHID));
  MatrixXd Rb = MatrixXd(random_embedding_mat(NC, 2 * KHID));
  MatrixXd Ra = MatrixXd(random_embedding_mat(NA, 2 * KHID));
  // rand() state now equals the one tensorDecom_alpha0 starts from
  MatrixXd A_random(MatrixXd::Random(KHID, KHID));
  A_random.setRandom();
  HouseholderQR<MatrixXd> qr(A_random);
  MatrixXd phi0 = qr.householderQ();
  // restore the same state before the real call
  { MatrixXd tmp = MatrixXd(random_embedding_mat(NA, 2 * KHID)); (void)tmp; }

  double t3 = now_s();
  VectorXd lambda(KHID);
  MatrixXd phi(KHID, KHID);
  tensorDecom_alpha0(Da, Da_mu, Db, Db_mu, Dc, Dc_mu, lambda, phi);
  double t4 = now_s();
  fprintf(tf, "stpm %.6f\n", t4 - t3);

  // post-processing (CommunityDetection.cpp:98-139)
  MatrixXd Inv_Lambda = (pinv_vector(lambda)).asDiagonal();
  SparseMatrix<double> inv_lam_phi = (Inv_Lambda.transpose() * phi.transpose()).sparseView();
  SparseMatrix<double> pi_tmp1 = inv_lam_phi * W.transpose();
  SparseMatrix<double> spi_a = (pi_tmp1 * Zb1) * Zb2 * Gb_a;
  SparseMatrix<double> spi_b = pi_tmp1 * Gb_a.transpose();
  SparseMatrix<double> spi_c = pi_tmp1 * Gc_a.transpose();
  SparseMatrix<double> spi_x = pi_tmp1 * Gx_a.transpose();
  MatrixXd pi_a = MatrixXd(spi_a), pi_b = MatrixXd(spi_b), pi_c = MatrixXd(spi_c), pi_x = MatrixXd(spi_x);
  long L = (long)NX + NA + NB + NC;
  MatrixXd pi_raw(KHID, L);
  pi_raw << pi_x, pi_a, pi_b, pi_c;
  MatrixXd pi = normProbMatrix(pi_raw);
  double t5 = now_s();
  fprintf(tf, "post %.6f\n", t5 - t4);
  fclose(tf);

  SparseMatrix<double> pi_sparse = pi.sparseView();
  write_pi((char*)(out + "/pi.txt").c_str(), pi_sparse);
  write_pi((char*)(out + "/white.txt").c_str(), W);

  dump(out + "/mu_a.txt", mu_a);
  dump(out + "/mu_b.txt", mu_b);
  dump(out + "/mu_c.txt", mu_c);
  dump(out + "/R_c.txt", Rc);
  dump(out + "/R_b.txt", Rb);
  dump(out + "/R_a.txt", Ra);
  dump(out + "/W.txt", MatrixXd(W));
  dump(out + "/Zb1.txt", MatrixXd(Zb1));
  dump(out + "/Zb2.txt", MatrixXd(Zb2));
  dump(out + "/Zc1.txt", MatrixXd(Zc1));
  dump(out + "/Zc2.txt", MatrixXd(Zc2));
  dump(out + "/Da.txt", MatrixXd(Da));
  dump(out + "/Db.txt", MatrixXd(Db));
  dump(out + "/Dc.txt", MatrixXd(Dc));
  dump(out + "/Da_mu.txt", Da_mu);
  dump(out + "/Db_mu.txt", Db_mu);
  dump(out + "/Dc_mu.txt", Dc_mu);
  dump(out + "/phi0.txt", phi0);
  dump(out + "/lambda.txt", lambda);
  dump(out + "/phi.txt", phi);
  dump(out + "/pi_raw.txt", pi_raw);
  dump(out + "/pi.txt.dense", pi);

  // one reference SGD step on sample 0 (Util.cpp:257-304) from Phi0
  VectorXd a0 = MatrixXd(Da).col(0), b0 = MatrixXd(Db).col(0), c0 = MatrixXd(Dc).col(0);
  MatrixXd step = Diff_Loss(a0, b0, c0, Da_mu, Db_mu, Dc_mu, phi0, 1e-7);
  dump(out + "/diffloss_phi.txt", step);
  VectorXd t2nd = The_second_term(a0, b0, c0, Da_mu, Db_mu, Dc_mu, phi0.col(0));
  dump(out + "/second_term.txt", t2nd);

  // normProbMatrix edge cases (Probability.cpp:33-121)
  MatrixXd edge(4, 5);
  edge << 0, 1.0, -3.0, 0.5, -1.0,
          0, -0.5, 1.0, 0.5, 2.0,
          0, 2.0, -1.0, -1.0, -1.0,
          0, 0.0, 0.5, 0.0, 0.0;
  dump(out + "/normprob_in.txt", edge);
  dump(out + "/normprob_out.txt", normProbMatrix(edge));
  return 0;
}

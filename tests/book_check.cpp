// Host harness of the per-iteration bookkeeping (m-themes_gb300/csrc/book.cuh):
// deterministic pseudo-random step constants and reduced sums, one call of
// book_finish then book_more / book_add, inputs and outputs printed as one
// JSON object per case for tests/test_book_host.py.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include "book.cuh"

using mth::IterBook;
constexpr int NP = 16;   // reduced sums of an iteration: err_s, err_e, sig[6], sig_ph1[6], Newton steps, failed solves

static uint64_t rng = 0x9e3779b97f4a7c15ULL;
static double urand() {   // [0, 1)
  rng ^= rng << 13;
  rng ^= rng >> 7;
  rng ^= rng << 17;
  return (double)(rng >> 11) * (1.0 / 9007199254740992.0);
}
static double srand1() { return 2.0 * urand() - 1.0; }

static void arr(const char* name, const double* v, int n, bool comma = true) {
  printf("\"%s\": [", name);
  for (int i = 0; i < n; i++) {   // JSON as Python reads it: NaN for a non-finite value
    if (std::isfinite(v[i])) printf("%.17g", v[i]);
    else printf("NaN");
    printf("%s", i + 1 < n ? ", " : "");
  }
  printf("]%s", comma ? ", " : "");
}
static void iarr(const char* name, const int* v, int n) {
  printf("\"%s\": [", name);
  for (int i = 0; i < n; i++) printf("%d%s", v[i], i + 1 < n ? ", " : "");
  printf("], ");
}

int main() {
  for (int c = 0; c < 12; c++) {
    IterBook b = {};
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) {
        b.udot[i][j] = srand1();
        b.scauchy[i][j] = 100.0 * srand1();
        b.ddg[i][j] = 1e-4 * srand1();
        b.ddg_acum[i][j] = 1e-3 * srand1();
        b.ddg_applied[i][j] = 1e-3 * srand1();
      }
    for (int k = 0; k < 81; k++) b.s0_4[k] = 1e-5 * srand1();
    for (int a = 0; a < 6; a++) {   // velocity or stress control per component
      b.vbc[a] = (c + a) % 3 != 0;
      b.sbc[a] = 1 - b.vbc[a];
    }
    b.wgt = 1.0 / (1000.0 + 100.0 * c);
    b.wgt_ph1 = b.wgt * (1.0 + 0.1 * urand());
    b.dt = 1e-3;
    b.err = 1e-5;
    b.e_vm = c % 4 == 0 ? 1e-6 : 1e-3 * (1.0 + urand());   // below 1e-5: Err_e set to 0
    b.iter_max = c % 5 == 0 ? 1 : 100;
    b.it_iter = c % 3;
    b.it_nit = 10 * c;
    b.it_nbad = c;
    double red[NP];
    for (int i = 0; i < NP; i++) red[i] = 1e3 * srand1();
    red[0] = fabs(red[0]) * 1e-2;
    red[1] = fabs(red[1]) * 1e-5;
    red[14] = (double)(int)(1e5 * urand());
    red[15] = (double)(c % 2);
    if (c == 7) red[9] = std::nan("");   // a non-finite sum
    printf("{");
    arr("udot", &b.udot[0][0], 9);
    arr("scauchy", &b.scauchy[0][0], 9);
    arr("s0_4", b.s0_4, 81);
    iarr("vbc", b.vbc, 6);
    iarr("sbc", b.sbc, 6);
    printf("\"wgt\": %.17g, \"wgt_ph1\": %.17g, \"dt\": %.17g, \"err\": %.17g, \"e_vm\": %.17g, \"iter_max\": %d, ",
           b.wgt, b.wgt_ph1, b.dt, b.err, b.e_vm, b.iter_max);
    printf("\"it_iter\": %d, \"it_nit\": %lld, \"it_nbad\": %lld, ", b.it_iter, b.it_nit, b.it_nbad);
    arr("ddg0", &b.ddg[0][0], 9);
    arr("ddg_acum0", &b.ddg_acum[0][0], 9);
    arr("ddg_applied0", &b.ddg_applied[0][0], 9);
    arr("red", red, NP);
    const bool ok = mth::book_finish(b, red, NP);
    double add[6] = {0, 0, 0, 0, 0, 0};
    int more = 0;
    if (ok) {
      more = mth::book_more(b);
      if (more) mth::book_add(b, add);
    }
    printf("\"ok\": %d, \"nan\": %d, \"more\": %d, ", (int)ok, b.nan, more);
    printf("\"out_it_iter\": %d, \"out_it_nit\": %lld, \"out_it_nbad\": %lld, ", b.it_iter, b.it_nit, b.it_nbad);
    arr("sig_avg", &b.sig_avg[0][0], 9);
    arr("sig_avg1", &b.sig_avg1[0][0], 9);
    arr("ddg", &b.ddg[0][0], 9);
    arr("ddg_acum", &b.ddg_acum[0][0], 9);
    arr("ddg_applied", &b.ddg_applied[0][0], 9);
    printf("\"err_s\": %.17g, \"err_e\": %.17g, \"s_vm\": %.17g, \"s_vm1\": %.17g, ", b.err_s, b.err_e, b.s_vm, b.s_vm1);
    arr("add", add, 6, false);
    printf("}\n");
  }
  return 0;
}

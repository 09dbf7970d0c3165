// Test driver: the host library's exact introsort against std::sort on the
// same (cell, elevation) pairs.  Returns the number of cases whose
// permutation differs.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <random>
#include <utility>
#include <vector>

void host_sort_exact(std::pair<double, double>* a, size_t n, int threads);

static int check(const std::vector<double>& v, int threads) {
  std::vector<std::pair<double, double>> a(v.size()), b;
  for (size_t k = 0; k < v.size(); k++) a[k] = std::make_pair((double)k, v[k]);
  b = a;
  std::sort(b.begin(), b.end(), [](const std::pair<double, double>& x,
                                   const std::pair<double, double>& y) {
    return x.second < y.second;
  });
  host_sort_exact(a.data(), a.size(), threads);
  for (size_t k = 0; k < a.size(); k++)
    if (a[k].first != b[k].first) return 1;
  return 0;
}

int main() {
  std::mt19937_64 rng(7);
  int bad = 0, cases = 0;
  const size_t sizes[] = {0, 1, 2, 15, 16, 17, 33, 100, 1000, 5000, 70000, 300000, 1200000};
  for (size_t n : sizes) {
    for (int kind = 0; kind < 7; kind++) {
      std::vector<double> v(n);
      for (size_t k = 0; k < n; k++) {
        switch (kind) {
          case 0: v[k] = (double)(rng() % 1000000) * 1e-3; break;       // few ties
          case 1: v[k] = (double)(rng() % 7); break;                     // heavy ties
          case 2: v[k] = (double)k; break;                               // sorted
          case 3: v[k] = (double)(n - k); break;                         // reversed
          case 4: v[k] = 5.0; break;                                     // all equal
          case 5: v[k] = (double)(k < n / 2 ? k : n - k); break;         // organ pipe
          default: v[k] = (k % 97 == 0) ? -9999.0 : 100 + (double)(rng() % 50) * 0.5;
        }
      }
      for (int t : {1, 4, 16}) {
        bad += check(v, t);
        cases++;
      }
    }
  }
  // inputs shaped like the reference's pair vector: (0, 0) padding around a
  // DEM with no-data cells and flats
  for (int rep = 0; rep < 4; rep++) {
    const int imax = 300 + rep * 17, jmax = 250 + rep * 11;
    std::vector<double> v((size_t)(imax + 2) * (jmax + 2), 0.0);
    size_t inc = 1;
    for (int i = 1; i <= imax; i++)
      for (int j = 1; j <= jmax; j++)
        v[inc++] = (j < 20 || (i + j) % 131 == 0) ? -9999.0 : 50 + 0.01 * (int)((i * 3 + j) / 4);
    for (int t : {1, 16}) {
      bad += check(v, t);
      cases++;
    }
  }
  // McIlroy's adversary ("A Killer Adversary for Quicksort", 1999) builds
  // inputs that drive median-of-three quicksort to its depth limit, so the
  // heapsort branch is exercised too
  for (size_t n : {2000, 50000}) {
    const long gas = (long)n;
    std::vector<long> val(n, gas);
    long nsolid = 0;
    size_t candidate = 0;
    std::vector<size_t> idx(n);
    for (size_t k = 0; k < n; k++) idx[k] = k;
    std::sort(idx.begin(), idx.end(), [&](size_t x, size_t y) {
      if (val[x] == gas && val[y] == gas) {
        if (x == candidate) val[x] = nsolid++;
        else val[y] = nsolid++;
      }
      if (val[x] == gas) candidate = x;
      else if (val[y] == gas) candidate = y;
      return val[x] < val[y];
    });
    for (size_t k = 0; k < n; k++)
      if (val[k] == gas) val[k] = nsolid++;
    std::vector<double> v(n);
    for (size_t k = 0; k < n; k++) v[k] = (double)val[k];
    for (int t : {1, 8}) {
      bad += check(v, t);
      cases++;
    }
  }
  printf("%d of %d cases differ\n", bad, cases);
  return bad;
}

// Checks thea::select_nth (thea_gb300/csrc/select_nth.cuh) against this C++ library's std::nth_element: the same
// permutation, element for element, on random arrays with and without ties, sorted and reversed arrays, and arrays
// built by M. D. McIlroy's adversary ("A Killer Adversary for Quicksort", 1999) to drive the selection into its
// heap-selection fallback. Elements carry a tag so that the order of equal keys is compared too.
#include "../../thea_gb300/csrc/select_nth.cuh"

#include <algorithm>
#include <cstdio>
#include <numeric>
#include <random>
#include <vector>

namespace {

struct Tagged {
  double key;
  int tag;
  bool operator<(Tagged const & o) const { return key < o.key; }
};

bool same_permutation(std::vector<double> const & keys, int nth) {
  std::vector<Tagged> a(keys.size());
  for (size_t i = 0; i < keys.size(); ++i) a[i] = Tagged{keys[i], (int)i};
  std::vector<Tagged> b = a;
  std::nth_element(a.begin(), a.begin() + nth, a.end());
  thea::select_nth(b.data(), (int)b.size(), nth);
  for (size_t i = 0; i < a.size(); ++i)
    if (a[i].tag != b[i].tag) return false;
  std::vector<double> c = keys, d = keys;  // plain doubles, as ShapeDiameter uses them
  std::nth_element(c.begin(), c.begin() + nth, c.end());
  thea::select_nth(d.data(), (int)d.size(), nth);
  return c == d;
}

// McIlroy's adversary: keys stay undecided ("gas") until a comparison needs them, then take the next value in
// increasing order, choosing the element the selection seems to use as its pivot candidate
std::vector<double> adversarial(int n, int nth) {
  int const GAS = n;
  std::vector<int> val(n, GAS);
  int solid = 0, candidate = 0;
  std::vector<int> idx(n);
  std::iota(idx.begin(), idx.end(), 0);
  auto cmp = [&](int x, int y) {
    if (val[x] == GAS && val[y] == GAS) {
      if (x == candidate) val[x] = solid++;
      else val[y] = solid++;
    }
    if (val[x] == GAS) candidate = x;
    else if (val[y] == GAS) candidate = y;
    return val[x] < val[y];
  };
  std::nth_element(idx.begin(), idx.begin() + nth, idx.end(), cmp);
  std::vector<double> keys(n);
  for (int i = 0; i < n; ++i) keys[i] = val[i] == GAS ? (double)(solid++) : (double)val[i];
  return keys;
}

}  // namespace

int main() {
  std::mt19937 rng(20240607u);
  long cases = 0;
  for (int n = 1; n <= 40; ++n) {
    for (int nth = 0; nth < n; ++nth) {
      std::vector<std::vector<double>> inputs;
      inputs.push_back(adversarial(n, nth));
      std::vector<double> sorted(n), reversed(n), organ(n);
      for (int i = 0; i < n; ++i) {
        sorted[i] = i;
        reversed[i] = n - i;
        organ[i] = std::min(i, n - 1 - i);
      }
      inputs.push_back(sorted);
      inputs.push_back(reversed);
      inputs.push_back(organ);
      for (int r = 0; r < 60; ++r) {
        std::vector<double> v(n);
        int distinct = r % 3 == 0 ? 3 : (r % 3 == 1 ? n : 1000000);
        std::uniform_int_distribution<int> u(0, distinct - 1);
        for (double & x : v) x = u(rng) * 0.25;
        inputs.push_back(v);
      }
      for (auto const & v : inputs) {
        ++cases;
        if (!same_permutation(v, nth)) {
          std::printf("mismatch: n=%d nth=%d\n", n, nth);
          return 1;
        }
      }
    }
  }
  std::printf("select_nth matches std::nth_element on %ld arrays\n", cases);
  return 0;
}

// Host-side check of the hierarchy builders (no GPU calls): on random
// scenes of instanced meshes (some with zero or one triangle), the flat and
// the two-level SAH topologies must be valid binary trees over every
// triangle -- perm a permutation, every internal node and leaf slot reached
// once from the root, parent links consistent -- and the two-level tree must
// keep each instance's triangles in one subtree.
#include "bvh.cu"

#include <cstdio>
#include <random>

namespace drgb {
void count_launch(int) {}
}  // namespace drgb

using namespace drgb;

static int check_tree(const std::vector<float4>& links, const std::vector<int>& perm, const std::vector<int>& lp,
                      const std::vector<int>& np, int n) {
  std::vector<int> seen_leaf(n, 0), seen_node(std::max(n - 1, 1), 0), seen_tri(n, 0);
  for (int k = 0; k < n; k++) {
    if (perm[k] < 0 || perm[k] >= n) return 1;
    if (seen_tri[perm[k]]++) return 2;
  }
  if (n < 2) return 0;
  if (np[0] != -1) return 3;
  std::vector<int> st{0};
  while (!st.empty()) {
    const int v = st.back();
    st.pop_back();
    if (v < 0 || v >= n - 1) return 4;
    if (seen_node[v]++) return 5;
    int c[2];
    std::memcpy(&c[0], &links[v].x, 4);
    std::memcpy(&c[1], &links[v].y, 4);
    for (int s = 0; s < 2; s++) {
      if (c[s] >= 0) {
        if (np[c[s]] != v) return 6;
        st.push_back(c[s]);
      } else {
        const int l = ~c[s];
        if (l >= n) return 7;
        if (seen_leaf[l]++) return 8;
        if (lp[l] != v) return 9;
      }
    }
  }
  for (int v = 0; v < n - 1; v++)
    if (!seen_node[v]) return 10;
  for (int l = 0; l < n; l++)
    if (!seen_leaf[l]) return 11;
  return 0;
}

// The leaf slots of one instance's triangles are contiguous (a subtree).
static int check_instances(const std::vector<int>& perm, const std::vector<int4>& tri_v, int n) {
  std::vector<int> first(4096, -1), last(4096, -1), count(4096, 0);
  for (int k = 0; k < n; k++) {
    const int b = tri_v[perm[k]].w;
    if (first[b] < 0) first[b] = k;
    last[b] = k;
    count[b]++;
  }
  for (int b = 0; b < 4096; b++)
    if (count[b] && last[b] - first[b] + 1 != count[b]) return 12;
  return 0;
}

int main() {
  std::mt19937 rng(1);
  int fails = 0, trees = 0;
  for (int trial = 0; trial < 300; trial++) {
    const int nm = 1 + rng() % 4;
    std::vector<BlockDev> blocks;
    std::vector<int4> tri_v;
    std::vector<float4> pos;
    std::vector<float> btr;
    int voff = 0, toff = 0;
    for (int m = 0; m < nm; m++) {
      const int nt = (rng() % 5 == 0) ? (int)(rng() % 2) : 1 + (int)(rng() % 200);
      const int nv = nt + 2;
      const int ninst = 1 + rng() % 6;
      std::vector<float4> local(nv);
      for (auto& p : local)
        p = make_float4((rng() % 1000) / 1000.f, (rng() % 1000) / 1000.f, (rng() % 1000) / 1000.f, 0.f);
      for (int j = 0; j < ninst; j++) {
        const int b = (int)blocks.size();
        blocks.push_back(BlockDev{voff, toff, m, j});
        const float off[3] = {(float)(rng() % 10), (float)(rng() % 10), (float)(rng() % 10)};
        for (auto p : local) pos.push_back(make_float4(p.x + off[0], p.y + off[1], p.z + off[2], 0.f));
        for (int t = 0; t < nt; t++) tri_v.push_back(make_int4(voff + t, voff + t + 1, voff + t + 2, b));
        std::vector<float> M(32, 0.f);
        M[0] = M[5] = M[10] = M[15] = 1.f;
        if (rng() % 2) {  // a quarter turn about z and a shift, applied twice when traced
          M[12] = 0.5f;
          M[0] = 0.f;
          M[1] = 1.f;
          M[4] = -1.f;
          M[5] = 0.f;
        }
        btr.insert(btr.end(), M.begin(), M.end());
        voff += nv;
        toff += nt;
      }
    }
    const int n = toff;
    if (n < 2) continue;
    std::vector<float4> links;
    std::vector<int> perm, lp, np;
    for (int builder : {1, 2, 3}) {
      host_topology(builder, pos.data(), btr.data(), tri_v, blocks, voff, n, links, perm, lp, np);
      int r = check_tree(links, perm, lp, np, n);
      if (!r && builder == 2) r = check_instances(perm, tri_v, n);
      trees++;
      if (r) {
        std::printf("trial %d builder %d: check %d failed (n=%d, blocks=%zu)\n", trial, builder, r, n, blocks.size());
        fails++;
      }
    }
  }
  std::printf("%d trees checked, %d failed\n", trees, fails);
  return fails != 0;
}

// A caller written against the reference's C++ API (uni10.hpp): U(1) bonds,
// UniTensor construction, setElem, permute, contract, Network::launch from a
// .net file, Block::svd and Block::eigh, save.  tests/test_cpp_driver.py
// compiles it against include/ and libtrim_gb300.so (a compile-and-link check
// on any machine) and, on a GPU, runs it and checks every saved result
// against the oracle.
//
// usage: drop_in_driver OUTDIR
#include <uni10.hpp>

#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

using namespace uni10;

static std::vector<Qnum> charges(const std::vector<int>& q, const std::vector<int>& deg) {
  std::vector<Qnum> out;
  for (size_t i = 0; i < q.size(); i++)
    for (int d = 0; d < deg[i]; d++) out.push_back(Qnum(q[i]));
  return out;
}

static void fill(UniTensor& t, double phase) {
  std::vector<double> e(t.elemNum());
  for (size_t i = 0; i < e.size(); i++) e[i] = std::sin(phase + 0.37 * (double)i);
  t.setElem(e);
}

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: %s OUTDIR\n", argv[0]);
    return 2;
  }
  const std::string dir = argv[1];
  try {
    std::vector<Qnum> qv = charges({-1, 0, 1}, {2, 3, 2});
    std::vector<Qnum> qp = charges({-1, 1}, {1, 1});
    Bond v_in(BD_IN, qv), v_out(BD_OUT, qv), p_in(BD_IN, qp);
    std::vector<Bond> a_bonds = {v_in, p_in, v_out};  // A[a, s | b]
    int la[] = {1, 2, 3};
    UniTensor A(a_bonds, la, "A");
    fill(A, 0.1);
    std::vector<Bond> b_bonds = {v_in, p_in, v_out};  // B[b, t | c]
    std::vector<int> lb = {3, 4, 5};
    UniTensor B(b_bonds, lb, "B");
    fill(B, 0.7);
    A.save(dir + "/A.bin");
    B.save(dir + "/B.bin");

    UniTensor AB = contract(A, B, false);  // over label 3
    AB.save(dir + "/AB.bin");

    UniTensor P = A;
    std::vector<int> np = {2, 1, 3};
    P.permute(np, 2);
    P.save(dir + "/PA.bin");

    {
      std::FILE* f = std::fopen((dir + "/chain.net").c_str(), "w");
      std::fprintf(f, "A: 1 2; 3\nB: 3 4; 5\nTOUT: 1 2 4; 5\nORDER: (A B)\n");
      std::fclose(f);
    }
    Network net(dir + "/chain.net");
    net.putTensor("A", A);
    net.putTensor("B", B);
    UniTensor N = net.launch();
    N.save(dir + "/NET.bin");

    // Block::svd and Block::eigh of the charge-0 block (9 x 9) of M[a | b]
    std::vector<Qnum> qm = charges({-1, 0, 1}, {4, 9, 4});
    std::vector<Bond> m_bonds = {Bond(BD_IN, qm), Bond(BD_OUT, qm)};
    UniTensor M(m_bonds, "M");
    fill(M, 1.3);
    M.save(dir + "/M.bin");
    Matrix blk = M.getBlock(Qnum(0));
    std::vector<Matrix> usv = blk.svd();
    std::vector<Matrix> ev = blk.eigh();
    std::FILE* f = std::fopen((dir + "/blocks.txt").c_str(), "w");
    std::vector<double> s = usv[1].hostElem(), e = ev[0].hostElem();
    std::fprintf(f, "rows %zu cols %zu\n", blk.row(), blk.col());
    for (double x : s) std::fprintf(f, "s %.17g\n", x);
    for (double x : e) std::fprintf(f, "e %.17g\n", x);
    std::fclose(f);
  } catch (const std::exception& ex) {
    std::fprintf(stderr, "driver: %s\n", ex.what());
    return 1;
  }
  std::printf("driver ok\n");
  return 0;
}

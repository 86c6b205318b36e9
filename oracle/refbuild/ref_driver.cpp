// Script-driven front end to the reference library's CPU path, compiled
// against the reference headers and linked with oracle/_ref/libuni10_ref.so.
// It is test infrastructure: it produces golden outputs for the parity tests
// and CPU timings for the baseline.  Nothing in the product links it.
//
// Script lines (whitespace separated; '#' starts a comment):
//   tensor NAME NBONDS             followed by NBONDS lines:
//     bond in|out NQ  (U1 PRT PRTF DEG) x NQ
//   labels NAME l0 l1 ...          UniTensor::setLabel
//   elems NAME PATH OFFSET         UniTensor::setElem from raw little-endian f64
//   permute NAME ROWNUM l0 l1 ...  UniTensor::permute(labels, rowBondNum)
//   permute_rows NAME ROWNUM       UniTensor::permute(rowBondNum)
//   transpose NAME                 UniTensor::transpose
//   contract OUT A B FAST          contract(A, B, fast)
//   otimes OUT A B                 otimes(A, B)
//   combine NAME l0 l1 ...         UniTensor::combineBond(labels)
//   network OUT NETFILE N1 T1 N2 T2 ...   Network::putTensor(Ni, Ti); launch()
//   copy OUT SRC                   deep copy
//   save NAME PATH                 UniTensor::save (current binary layout)
//   name NAME STR                  UniTensor::setName
//   svd NAME U1 PRT PRTF PREFIX    Block::svd of one block -> PREFIX.{U,S,VT}
//   eigh NAME U1 PRT PRTF PREFIX   Block::eigh of one block -> PREFIX.{E,V}
//   addgate NAME B1 B2 [B1 B2 ...]  UniTensor::addGate with these bond swaps
//   blocks NAME PATH               writes "U1 PRT PRTF ROWS COLS" per block
//   time ITERS <command...>        runs the command ITERS times (on copies
//                                  for in-place ones) and prints seconds/iter
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include <uni10.hpp>

using namespace uni10;

static std::map<std::string, UniTensor> T;

static std::vector<std::string> split(const std::string& s) {
  std::istringstream is(s);
  std::vector<std::string> out;
  std::string w;
  while (is >> w) {
    if (w[0] == '#') break;
    out.push_back(w);
  }
  return out;
}

static UniTensor& get(const std::string& n) {
  auto it = T.find(n);
  if (it == T.end()) {
    std::cerr << "ref_driver: unknown tensor " << n << std::endl;
    std::exit(3);
  }
  return it->second;
}

static std::vector<int> ints(const std::vector<std::string>& w, size_t from) {
  std::vector<int> v;
  for (size_t i = from; i < w.size(); i++) v.push_back(std::atoi(w[i].c_str()));
  return v;
}

static void run(const std::vector<std::string>& w);

static void run_timed(const std::vector<std::string>& w) {
  int iters = std::atoi(w[1].c_str());
  std::vector<std::string> cmd(w.begin() + 2, w.end());
  const std::string& op = cmd[0];
  // in-place operations run on a fresh copy each iteration; the copy is
  // taken outside the timed region.
  bool inplace = (op == "permute" || op == "permute_rows" || op == "transpose" || op == "combine");
  double total = 0;
  for (int i = 0; i < iters + 1; i++) {
    std::vector<std::string> c = cmd;
    if (inplace) {
      T["__timed"] = get(cmd[1]);
      c[1] = "__timed";
    }
    if (op == "contract") {
      T["__ta"] = get(cmd[2]);
      T["__tb"] = get(cmd[3]);
      c[2] = "__ta";
      c[3] = "__tb";
    }
    auto t0 = std::chrono::steady_clock::now();
    run(c);
    auto t1 = std::chrono::steady_clock::now();
    if (i > 0) total += std::chrono::duration<double>(t1 - t0).count();  // first is warm-up
  }
  std::printf("time %s %.9e\n", op.c_str(), total / iters);
  std::fflush(stdout);
}

static void run(const std::vector<std::string>& w) {
  const std::string& op = w[0];
  if (op == "permute") {
    get(w[1]).permute(ints(w, 3), std::atoi(w[2].c_str()));
  } else if (op == "permute_rows") {
    get(w[1]).permute(std::atoi(w[2].c_str()));
  } else if (op == "transpose") {
    get(w[1]).transpose();
  } else if (op == "contract") {
    UniTensor c = contract(get(w[2]), get(w[3]), std::atoi(w[4].c_str()) != 0);
    T[w[1]] = c;
  } else if (op == "otimes") {
    T[w[1]] = otimes(get(w[2]), get(w[3]));
  } else if (op == "combine") {
    get(w[1]).combineBond(ints(w, 2));
  } else if (op == "network") {
    Network net(w[2]);
    for (size_t i = 3; i + 1 < w.size(); i += 2) net.putTensor(w[i], get(w[i + 1]));
    T[w[1]] = net.launch();
  } else if (op == "copy") {
    T[w[1]] = get(w[2]);
  } else if (op == "save") {
    get(w[1]).save(w[2]);
  } else if (op == "name") {
    get(w[1]).setName(w[2]);
  } else if (op == "labels") {
    get(w[1]).setLabel(ints(w, 2));
  } else if (op == "svd") {
    Qnum q(parityFType(std::atoi(w[4].c_str())), std::atoi(w[2].c_str()), parityType(std::atoi(w[3].c_str())));
    std::vector<Matrix> r = get(w[1]).getBlock(q).svd();
    const char* suf[3] = {".U", ".S", ".VT"};
    for (int k = 0; k < 3; k++) {
      FILE* fp = std::fopen((w[5] + suf[k]).c_str(), "wb");
      size_t rc[2] = {r[k].row(), r[k].col()};
      std::fwrite(rc, sizeof(size_t), 2, fp);
      std::fwrite(r[k].getElem(), sizeof(double), r[k].elemNum(), fp);
      std::fclose(fp);
    }
  } else if (op == "addgate") {
    std::vector<_Swap> sw;
    for (size_t i = 2; i + 1 < w.size(); i += 2) {
      _Swap s;
      s.b1 = std::atoi(w[i].c_str());
      s.b2 = std::atoi(w[i + 1].c_str());
      sw.push_back(s);
    }
    get(w[1]).addGate(sw);
  } else if (op == "eigh") {
    Qnum q(parityFType(std::atoi(w[4].c_str())), std::atoi(w[2].c_str()), parityType(std::atoi(w[3].c_str())));
    std::vector<Matrix> r = get(w[1]).getBlock(q).eigh();
    const char* suf[2] = {".E", ".V"};
    for (int k = 0; k < 2; k++) {
      FILE* fp = std::fopen((w[5] + suf[k]).c_str(), "wb");
      size_t rc[2] = {r[k].row(), r[k].col()};
      std::fwrite(rc, sizeof(size_t), 2, fp);
      std::fwrite(r[k].getElem(), sizeof(double), r[k].elemNum(), fp);
      std::fclose(fp);
    }
  } else if (op == "blocks") {
    std::ofstream os(w[2].c_str());
    UniTensor& t = get(w[1]);
    std::vector<Qnum> qs = t.blockQnum();
    for (size_t i = 0; i < qs.size(); i++) {
      Matrix m = t.getBlock(qs[i]);
      os << qs[i].U1() << " " << int(qs[i].prt()) << " " << int(qs[i].prtF()) << " " << m.row() << " " << m.col()
         << "\n";
    }
  } else if (op == "time") {
    run_timed(w);
  } else {
    std::cerr << "ref_driver: unknown command " << op << std::endl;
    std::exit(2);
  }
}

int main(int argc, char** argv) {
  std::istream* in = &std::cin;
  std::ifstream f;
  if (argc > 1) {
    f.open(argv[1]);
    in = &f;
  }
  std::string line;
  while (std::getline(*in, line)) {
    std::vector<std::string> w = split(line);
    if (w.empty()) continue;
    if (w[0] == "tensor") {
      int nb = std::atoi(w[2].c_str());
      std::vector<Bond> bonds;
      for (int b = 0; b < nb; b++) {
        std::getline(*in, line);
        std::vector<std::string> bw = split(line);
        bondType tp = (bw[1] == "in") ? BD_IN : BD_OUT;
        int nq = std::atoi(bw[2].c_str());
        std::vector<Qnum> qlist;
        for (int q = 0; q < nq; q++) {
          int u1 = std::atoi(bw[3 + 4 * q].c_str());
          int prt = std::atoi(bw[4 + 4 * q].c_str());
          int prtf = std::atoi(bw[5 + 4 * q].c_str());
          int deg = std::atoi(bw[6 + 4 * q].c_str());
          Qnum qn(parityFType(prtf), u1, parityType(prt));
          for (int d = 0; d < deg; d++) qlist.push_back(qn);
        }
        bonds.push_back(Bond(tp, qlist));
      }
      T[w[1]] = UniTensor(bonds, w[1]);
    } else if (w[0] == "elems") {
      UniTensor& t = get(w[1]);
      std::vector<double> buf(t.elemNum());
      FILE* fp = std::fopen(w[2].c_str(), "rb");
      if (!fp) {
        std::cerr << "ref_driver: cannot open " << w[2] << std::endl;
        return 4;
      }
      std::fseek(fp, std::atol(w[3].c_str()), SEEK_SET);
      size_t got = std::fread(buf.data(), sizeof(double), buf.size(), fp);
      std::fclose(fp);
      if (got != buf.size()) {
        std::cerr << "ref_driver: short read for " << w[1] << std::endl;
        return 4;
      }
      t.setElem(buf.data());
    } else {
      run(w);
    }
  }
  return 0;
}

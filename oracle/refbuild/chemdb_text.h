// The species database of a reacting case for the golden-output harness
// (test infrastructure only).  The reference reads it from an HDF5 file
// (Species::GetDBInfo, ucs/species.tcc:140) that its Python builder writes;
// here <case>/chemdb.txt carries the same datasets as text (one per line:
// "species <name>", "<dataset> <value>" for scalars, "<dataset> <rows> <cols>
// <values...>" for arrays) and is written through the reference's own h5layer
// writers into <case>/chemdb.h5 (the stand-in file store), which the case's
// chemicalDatabase names.  Include after the reference's h5layer.h.
#ifndef PCFD_CHEMDB_TEXT_H__
#define PCFD_CHEMDB_TEXT_H__

#include <fstream>
#include <sstream>
#include <string>
#include <vector>

inline int write_chem_db(const std::string& dir) {
  std::ifstream in((dir + "chemdb.txt").c_str());
  if (!in.is_open()) return 0;
  hid_t f = HDF_CreateFile(dir + "chemdb.h5", 1);
  if (f < 0) return -1;
  std::string line, group;
  while (std::getline(in, line)) {
    std::istringstream ls(line);
    std::string key;
    if (!(ls >> key)) continue;
    if (key == "species") {
      std::string name;
      ls >> name;
      group = "/species/" + name;
      continue;
    }
    std::vector<double> v;
    double x;
    while (ls >> x) v.push_back(x);
    if (v.size() == 1) {
      HDF_WriteScalar(f, group, key, &v[0]);
    } else if (v.size() >= 2) {
      const int rows = (int)v[0], cols = (int)v[1];
      if ((size_t)rows * cols + 2 != v.size()) return -2;
      HDF_WriteArray(f, group, key, &v[2], rows, cols);
    }
  }
  HDF_CloseFile(f);
  return 0;
}

#endif

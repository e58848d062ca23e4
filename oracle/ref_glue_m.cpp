// ORACLE — test infrastructure only.  C-linkage entry point onto the
// reference's unweighted Newman modularity tool
// U/Newman_Modularity_CPU/Modularity_CPU/Modularity_CPU.cpp, compiled by
// build.py from the reference tree into oracle/_ref/ (its main() renamed and
// never called; its timer and Maslov rewiring are not used).
#include <iostream>
#include <set>

extern long long N;                                  // Modularity_CPU.cpp:22
extern double *v, *v0, *verr, *sumBG;                // :23
void Partition(int* R, int* C, int* Result);         // :173

void Setup(int) {}
void Start(int) {}
void Stop(int) {}
double GetElapsedTime(int) { return 0.0; }
void Maslov(int*, int*, int*, int*, int, int) {}

extern "C" int ref_m_partition(int* R, int* C, int n, int* result) {
  N = n;
  v = new double[n];
  v0 = new double[n];
  verr = new double[n];
  sumBG = new double[n];
  std::cout.setstate(std::ios::failbit);  // the tool prints its progress
  Partition(R, C, result);
  std::cout.clear();
  delete[] v;
  delete[] v0;
  delete[] verr;
  delete[] sumBG;
  std::set<int> labels(result, result + n);
  return (int)labels.size();
}

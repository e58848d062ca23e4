// ORACLE — test infrastructure only.  C-linkage entry points onto the
// reference's multi-threaded CPU correlation tool
// U/CorMat/CorMat_CPU/CorMat/CorMat_CPU.cpp, compiled by build.py from the
// reference tree into oracle/_ref/ (Win32 threads mapped by refshim/).
typedef float real__t;
extern int numThread;                                                     // CorMat_CPU.cpp:20
void CorMat_cpu(real__t* Cormat, real__t* BOLD, int N, int L);            // :229
void CorMat_cpu_MT(real__t* Cormat, real__t* BOLD, int N, int L);         // :283
int FormFullGraph(bool* adjacent, real__t* Cormat, int N, real__t threshold);  // :190
void FormCSRGraph(int* R, int* C, bool* adjacent, int N);                 // :209

extern "C" {
void ref_u_cormat_cpu_mt(float* Cormat, float* BOLD, int N, int L, int threads) {
  numThread = threads > 0 ? threads : 1;
  CorMat_cpu_MT(Cormat, BOLD, N, L);
}
void ref_u_cormat_cpu(float* Cormat, float* BOLD, int N, int L) { CorMat_cpu(Cormat, BOLD, N, L); }
int ref_u_form_full_graph(bool* adj, float* Cormat, int N, float thr) {
  return FormFullGraph(adj, Cormat, N, thr);
}
void ref_u_form_csr_graph(int* R, int* C, bool* adj, int N) { FormCSRGraph(R, C, adj, N); }
}

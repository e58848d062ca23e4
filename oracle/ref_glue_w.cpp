// ORACLE — test infrastructure only.  C-linkage entry points onto the
// reference's own CPU functions of W/CorMat/CUCorMat/CUCorMat/CorMat.cpp,
// which build.py compiles from the reference tree into oracle/_ref/.
// The GPU symbols that file's main() refers to get inert stubs here; main()
// itself is renamed at compile time and never called.
typedef float real__t;

void CorMat_cpu(real__t* Cormat, real__t* BOLD, int N, int L);            // CorMat.cpp:921
long long FormFullGraph(bool* adjacent, real__t* Cormat, int N, real__t threshold);  // :683
real__t FormFullGraph_s(bool* adjacent, real__t* Cormat, int N, long long threshold);  // :743
void post_block(real__t* Cormat, real__t* Cormat_blocked, int dim, int block_size,
                bool fishtran_flag);                                           // :824
void FormCSRGraph(int* R, int* C, real__t* V, bool* adjacent, int N, real__t* Cormat);  // :889

int CorMat_gpu(real__t*, real__t*, int, int, int) { return -1; }
long long find_max(real__t*, long long) { return -1; }
real__t select_GPU(real__t*, long long, long long) { return 0; }

extern "C" {
void ref_w_cormat_cpu(float* Cormat, float* BOLD, int N, int L) { CorMat_cpu(Cormat, BOLD, N, L); }
long long ref_w_form_full_graph(bool* adj, float* Cormat, int N, float thr) {
  return FormFullGraph(adj, Cormat, N, thr);
}
float ref_w_form_full_graph_s(bool* adj, float* Cormat, int N, long long k) {
  return FormFullGraph_s(adj, Cormat, N, k);
}
void ref_w_form_csr_graph(int* R, int* C, float* V, bool* adj, int N, float* Cormat) {
  FormCSRGraph(R, C, V, adj, N, Cormat);
}
void ref_w_post_block(float* Cormat, float* blocked, int N, int B, int fisher) {
  post_block(Cormat, blocked, N, B, fisher != 0);
}
}

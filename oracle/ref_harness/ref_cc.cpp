/* ref_cc <csr> <out.bin>  — runs the reference's serial CC program
 * (CC/serial/serial.cpp:119-227) unchanged and captures its label array.
 * The labels live in a local of the reference's main (serial.cpp:157) and are
 * released with free(value) (serial.cpp:221); every standard header is
 * included first, then `free` is redirected to og_ref_capture_free, which
 * copies the first block released (the labels) before the program drops it.
 * OG_REF_SRC is the path of the reference's serial.cpp. */
#include "ref_common.hpp"

static uint64_t og_ref_V = 0;
static std::vector<unsigned> og_ref_labels;
static int og_ref_frees = 0;
static void og_ref_capture_free(void *p) {
  if (og_ref_frees++ == 0)
    og_ref_labels.assign((unsigned *)p, (unsigned *)p + og_ref_V);
}

#define free og_ref_capture_free
#define main og_ref_main
#include OG_REF_SRC
#undef main
#undef free

int main(int argc, char **argv) {
  if (argc != 3) {
    fprintf(stderr, "usage: ref_cc <csr> <out.bin>\n");
    return 2;
  }
  og_ref_V = og_ref_read_vertex_count(argv[1]);
  char a0[] = "ref_cc", a1[] = "-f";
  char *args[] = {a0, a1, argv[1], nullptr};
  const double t0 = og_ref_now_ms();
  og_ref_main(3, args);
  const double ms = og_ref_now_ms() - t0;
  if (og_ref_labels.size() != og_ref_V) {
    fprintf(stderr, "label capture failed\n");
    return 3;
  }
  og_ref_write(argv[2], og_ref_labels.data(), sizeof(unsigned) * og_ref_V);
  fprintf(stderr, "ms %.3f\n", ms);
  return 0;
}

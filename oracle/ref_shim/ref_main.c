/* Entry point of the reference-as-oracle binary: runs the reference's own
 * main() (src/main.c:267, symbol renamed at build time). */
int goma_ref_main(int argc, char **argv);
int main(int argc, char **argv) { return goma_ref_main(argc, argv); }

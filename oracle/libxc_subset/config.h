/* Minimal configuration header for compiling the LDA_X + LDA_C_PW subset of
 * the vendored libxc 6.2.2 as a CPU checker.  Only the energy and first
 * derivative are needed, so the higher derivative kernels are left out. */
#define PACKAGE_VERSION "6.2.2"
#define XC_DONT_COMPILE_FXC 1
#define XC_DONT_COMPILE_KXC 1
#define XC_DONT_COMPILE_LXC 1

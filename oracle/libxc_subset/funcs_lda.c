/* Trimmed functional table: only Slater exchange (id 1) and Perdew-Wang 92
 * correlation (id 12) are registered.  Included by libxc's lda.c in place of
 * its full table (the build stages lda.c next to this file). */
extern xc_func_info_type xc_func_info_lda_x;
extern xc_func_info_type xc_func_info_lda_c_pw;
const xc_func_info_type *xc_lda_known_funct[] = {
  &xc_func_info_lda_x, &xc_func_info_lda_c_pw, NULL
};

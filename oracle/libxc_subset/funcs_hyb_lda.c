/* No hybrid LDA functionals in the checker subset. */
const xc_func_info_type *xc_hyb_lda_known_funct[] = { NULL };

/* Empty functional tables for the families the checker subset leaves out,
 * plus aborting stand-ins for the GGA/meta-GGA entry points that libxc's
 * mixing code references but the LDA subset never reaches. */
#include <stdio.h>
#include <stdlib.h>
typedef struct xc_func_info_type xc_func_info_type;
const xc_func_info_type *xc_gga_known_funct[] = { NULL };
const xc_func_info_type *xc_hyb_gga_known_funct[] = { NULL };
const xc_func_info_type *xc_mgga_known_funct[] = { NULL };
const xc_func_info_type *xc_hyb_mgga_known_funct[] = { NULL };
static void unreachable(const char *what) {
  fprintf(stderr, "libxc subset: %s is not part of the LDA checker\n", what);
  abort();
}
void xc_gga() { unreachable("xc_gga"); }
void xc_mgga() { unreachable("xc_mgga"); }
void xc_hyb_init_hybrid() { unreachable("xc_hyb_init_hybrid"); }
void xc_mgga_vars_allocate_all() { unreachable("xc_mgga_vars_allocate_all"); }
void xc_mgga_vars_free_all() { unreachable("xc_mgga_vars_free_all"); }

/* Version header normally generated by libxc's configure step (6.2.2). */
#ifndef _XC_VERSION_H
#define _XC_VERSION_H
#define XC_VERSION "6.2.2"
#define XC_MAJOR_VERSION 6
#define XC_MINOR_VERSION 2
#define XC_MICRO_VERSION 2
#endif

/* Only the BYTE typedef from the Win32 header is used by the reference
 * headers on the hot path.  Oracle build only. */
#ifndef WAP_REF_SHIM_WINDOWS_H
#define WAP_REF_SHIM_WINDOWS_H
typedef unsigned char BYTE;
#endif

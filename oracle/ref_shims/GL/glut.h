/* Headless stand-in for GLUT: the reference only needs the GL no-ops.
 * Oracle build only. */
#include "glew.h"

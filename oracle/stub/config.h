/* project-written configuration for compiling the reference sources as a test oracle */
#define PACKAGE "locarna"
#define PACKAGE_NAME "LocARNA"
#define PACKAGE_VERSION "2.0.1"
#define PACKAGE_STRING "LocARNA 2.0.1"
#define PACKAGE_TARNAME "locarna"
#define PACKAGE_URL ""
#define PACKAGE_BUGREPORT ""
#define VERSION "2.0.1"
#define HAVE_LIBRNA 1

/* The three values CMake writes into the reference's CMCConfig.h
 * (CMCConfig.h.in, CMakeLists.txt:21-23), for oracle/ref.mk. */
#define CMC_VERSION_MAJOR 1
#define CMC_VERSION_MINOR 0
#define CMCPRETTYNAME "ClusterMonteCarlo"

/* Stand-in for the OptiX SDK header, which this machine does not have.  The reference
 * sources compiled by oracle/ref_build.py only need the handle type from it. */
#pragma once
typedef unsigned long long OptixTraversableHandle;

/* Empty stand-in for plplot.h: the reference's ns_cube.h pulls in
   matrix_plot.h, which includes <plplot.h>, but the NSCube step uses none of
   it.  Test infrastructure only. */
#pragma once

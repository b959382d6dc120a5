/* C2A/src/InterpMotion.cpp:7 includes GLUT but uses none of it; no graphics here. */

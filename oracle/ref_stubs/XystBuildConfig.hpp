// Stand-in for the configure-time header of the reference build: selects the
// default node-major (unknown, component) field layout and nothing else.
#pragma once
#define FIELD_DATA_LAYOUT_AS_FIELD_MAJOR

// Stand-in for src/app/Utils.h: only RandomFloat is used by Dataset.cpp.
#pragma once
float RandomFloat(float min = 0.0f, float max = 1.0f);

// Linux shim for the reference's Timer.h (timing helpers of its CPU tools);
// the oracle glue defines them as no-ops.
#pragma once
void Setup(int n);
void Start(int n);
void Stop(int n);
double GetElapsedTime(int n);

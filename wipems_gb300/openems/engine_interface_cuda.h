// engine_interface_cuda.h -- Engine_Interface_CUDA: the field-access adapter
// openEMS's processing uses (Engine_Interface_FDTD, engine_interface_fdtd.h)
// for Engine_CUDA.  Voltage integrals and the energy estimate are computed
// on the device in one call each (fdtd_engine_probe_now, fdtd_engine_energy)
// instead of one device read per node; point fields (dumps, field probes,
// ProcessCurrent's loop) go through Engine_CUDA::GetVolt / GetCurr.
#ifndef ENGINE_INTERFACE_CUDA_H
#define ENGINE_INTERFACE_CUDA_H

#include "FDTD/engine_interface_fdtd.h"

class Engine_CUDA;

class Engine_Interface_CUDA : public Engine_Interface_FDTD
{
public:
	Engine_Interface_CUDA(Operator* op, Engine_CUDA* eng);
	virtual ~Engine_Interface_CUDA();

	//! Engine_Interface_FDTD::CalcVoltageIntegral (engine_interface_fdtd.cpp:200-226) on the device
	virtual double CalcVoltageIntegral(const unsigned int* start, const unsigned int* stop) const;
	//! Engine_Interface_FDTD::CalcFastEnergy (engine_interface_fdtd.cpp:292-337) on the device
	virtual double CalcFastEnergy() const;

protected:
	Engine_CUDA* m_EngCUDA;
};

#endif // ENGINE_INTERFACE_CUDA_H

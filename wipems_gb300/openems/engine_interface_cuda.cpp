// engine_interface_cuda.cpp -- Engine_Interface_CUDA (see engine_interface_cuda.h).
#include "engine_interface_cuda.h"

#include <iostream>

#include "engine_cuda.h"

Engine_Interface_CUDA::Engine_Interface_CUDA(Operator* op, Engine_CUDA* eng) : Engine_Interface_FDTD(op), m_EngCUDA(eng)
{
	SetFDTDEngine(eng);
}

Engine_Interface_CUDA::~Engine_Interface_CUDA()
{
}

double Engine_Interface_CUDA::CalcVoltageIntegral(const unsigned int* start, const unsigned int* stop) const
{
	fdtd_probe_desc p = {};
	p.type = 0;
	for (int n = 0; n < 3; ++n)
	{
		p.start[n] = start[n];
		p.stop[n] = stop[n];
		p.start_inside[n] = 1;
		p.stop_inside[n] = 1;
	}
	p.norm_dir = -1;
	p.weight = 1.0;
	p.enabled = 1;
	double v = 0;
	if (fdtd_engine_probe_now(m_EngCUDA->Handle(), &p, &v) != FDTD_OK)
	{
		char msg[512];
		fdtd_last_error(msg, sizeof(msg));
		std::cerr << "Engine_Interface_CUDA::CalcVoltageIntegral: " << msg << std::endl;
	}
	return v;
}

double Engine_Interface_CUDA::CalcFastEnergy() const
{
	double e = 0;
	if (fdtd_engine_energy(m_EngCUDA->Handle(), &e) != FDTD_OK)
	{
		char msg[512];
		fdtd_last_error(msg, sizeof(msg));
		std::cerr << "Engine_Interface_CUDA::CalcFastEnergy: " << msg << std::endl;
	}
	return e;
}

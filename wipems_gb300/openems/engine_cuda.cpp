// engine_cuda.cpp -- Engine_CUDA (see engine_cuda.h).
#include "engine_cuda.h"

#include <iostream>

#include "operator_cuda.h"

Engine_CUDA* Engine_CUDA::New(const Operator_CUDA* op)
{
	std::cout << "Create FDTD engine (GB300 CUDA)" << std::endl;
	Engine_CUDA* e = new Engine_CUDA(op);
	e->Init();
	return e;
}

Engine_CUDA::Engine_CUDA(const Operator_CUDA* op) : Engine(op), m_Op_CUDA(op), m_cop(0), m_eng(0)
{
	m_type = UNKNOWN;  // the extension dispatcher has no CUDA engine type: no engine extensions are made
}

Engine_CUDA::~Engine_CUDA()
{
	Engine_CUDA::Reset();
}

void Engine_CUDA::Fail(const char* where) const
{
	char msg[512];
	fdtd_last_error(msg, sizeof(msg));
	std::cerr << "Engine_CUDA: " << where << ": " << msg << std::endl;
}

void Engine_CUDA::Init()
{
	numTS = 0;
	wipems_openems::OperatorView view;
	if (!m_Op_CUDA->Describe(view))
		return;
	if (fdtd_compress(&view.desc, &m_cop) != FDTD_OK)
	{
		Fail("fdtd_compress");
		return;
	}
	fdtd_engine_opts opts = {};
	opts.device = 0;
	opts.use_graphs = 1;
	opts.energy_on_probe = 0;  // openEMS's processing evaluates probes and energy on its own schedule
	if (fdtd_engine_create_compressed(m_cop, &opts, &m_eng) != FDTD_OK)
	{
		Fail("fdtd_engine_create_compressed");
		m_eng = 0;
	}
}

void Engine_CUDA::Reset()
{
	if (m_eng)
		fdtd_engine_destroy(m_eng);
	if (m_cop)
		fdtd_cop_destroy(m_cop);
	m_eng = 0;
	m_cop = 0;
	numTS = 0;
}

bool Engine_CUDA::IterateTS(unsigned int iterTS)
{
	if (!m_eng)
		return false;
	if (fdtd_engine_iterate(m_eng, iterTS) != FDTD_OK)
	{
		Fail("IterateTS");
		return false;
	}
	uint32_t ts = 0;
	fdtd_engine_num_timesteps(m_eng, &ts);
	numTS = ts;
	return true;
}

FDTD_FLOAT Engine_CUDA::GetVolt(unsigned int n, unsigned int x, unsigned int y, unsigned int z) const
{
	float v = 0;
	if (!m_eng || fdtd_engine_get_volt(m_eng, n, x, y, z, &v) != FDTD_OK)
		Fail("GetVolt");
	return v;
}

FDTD_FLOAT Engine_CUDA::GetCurr(unsigned int n, unsigned int x, unsigned int y, unsigned int z) const
{
	float v = 0;
	if (!m_eng || fdtd_engine_get_curr(m_eng, n, x, y, z, &v) != FDTD_OK)
		Fail("GetCurr");
	return v;
}

void Engine_CUDA::SetVolt(unsigned int n, unsigned int x, unsigned int y, unsigned int z, FDTD_FLOAT value)
{
	if (!m_eng || fdtd_engine_set_volt(m_eng, n, x, y, z, value) != FDTD_OK)
		Fail("SetVolt");
}

void Engine_CUDA::SetCurr(unsigned int n, unsigned int x, unsigned int y, unsigned int z, FDTD_FLOAT value)
{
	if (!m_eng || fdtd_engine_set_curr(m_eng, n, x, y, z, value) != FDTD_OK)
		Fail("SetCurr");
}

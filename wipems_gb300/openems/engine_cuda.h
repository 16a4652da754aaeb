// engine_cuda.h -- Engine_CUDA: openEMS's Engine on the GB300 engine
// (libwipems_fdtd.so, include/wipems_fdtd.h).
//
// Engine::IterateTS (FDTD/engine.cpp:255-274) runs on the device: the E and
// H half-steps with the UPML, Lorentz/Drude, excitation, Mur and lumped RLC
// updates fused in, in the reference's hook order.  The fields live in GPU
// memory; GetVolt / GetCurr / SetVolt / SetCurr (engine.h:53-61) read and
// write single values there.  No engine extension objects are created: their
// updates are part of the device kernels, so the extension hooks of the base
// class are never called.
#ifndef ENGINE_CUDA_H
#define ENGINE_CUDA_H

#include "FDTD/engine.h"
#include "openems_bridge.h"
#include "wipems_fdtd.h"

class Operator_CUDA;

class Engine_CUDA : public Engine
{
public:
	static Engine_CUDA* New(const Operator_CUDA* op);
	virtual ~Engine_CUDA();

	//! Engine::Init: describe the operator, compress it and upload it to the
	//! device (fields zero, numTS = 0)
	virtual void Init();
	//! Engine::Reset: release the device engine
	virtual void Reset();

	//! Iterate a number of timesteps on the device (false on an engine error,
	//! with the message on stderr)
	virtual bool IterateTS(unsigned int iterTS);
	virtual unsigned int GetNumberOfTimesteps() {return numTS;}

	virtual FDTD_FLOAT GetVolt(unsigned int n, unsigned int x, unsigned int y, unsigned int z) const;
	virtual FDTD_FLOAT GetVolt(unsigned int n, const unsigned int pos[3]) const {return GetVolt(n, pos[0], pos[1], pos[2]);}
	virtual FDTD_FLOAT GetCurr(unsigned int n, unsigned int x, unsigned int y, unsigned int z) const;
	virtual FDTD_FLOAT GetCurr(unsigned int n, const unsigned int pos[3]) const {return GetCurr(n, pos[0], pos[1], pos[2]);}
	virtual void SetVolt(unsigned int n, unsigned int x, unsigned int y, unsigned int z, FDTD_FLOAT value);
	virtual void SetVolt(unsigned int n, const unsigned int pos[3], FDTD_FLOAT value) {SetVolt(n, pos[0], pos[1], pos[2], value);}
	virtual void SetCurr(unsigned int n, unsigned int x, unsigned int y, unsigned int z, FDTD_FLOAT value);
	virtual void SetCurr(unsigned int n, const unsigned int pos[3], FDTD_FLOAT value) {SetCurr(n, pos[0], pos[1], pos[2], value);}

	//! The device engine (probe integrals, energy, dumps through the C ABI)
	fdtd_engine_t Handle() const {return m_eng;}

protected:
	Engine_CUDA(const Operator_CUDA* op);
	const Operator_CUDA* m_Op_CUDA;
	fdtd_cop_t m_cop;
	fdtd_engine_t m_eng;
	void Fail(const char* where) const;
};

#endif // ENGINE_CUDA_H

// operator_cuda.h -- Operator_CUDA: openEMS's Operator for the GB300 engine.
//
// Built inside the openEMS tree.  The operator build is
// openEMS's own (Operator::CalcECOperator and the extensions' BuildExtension,
// FDTD/operator.cpp:973-1084); this class only creates the CUDA engine
// (Operator::CreateEngine, operator.h:55) and hands it the built arrays as
// the engine description of include/wipems_fdtd.h.
#ifndef OPERATOR_CUDA_H
#define OPERATOR_CUDA_H

#include "FDTD/operator.h"
#include "openems_bridge.h"

class Operator_CUDA : public Operator
{
public:
	//! Create a new operator (Operator::New, operator.cpp:40-45)
	static Operator_CUDA* New();
	virtual ~Operator_CUDA();

	//! Engine_CUDA on this operator (Operator::CreateEngine, operator.h:55)
	virtual Engine* CreateEngine();

	//! The engine description of the built operator and its UPML,
	//! Lorentz/Drude, excitation, Mur and lumped RLC extensions, flattened
	//! into host storage the view owns.  Call after CalcECOperator and after
	//! Excitation::buildExcitationSignal.  False if an extension the CUDA
	//! engine does not provide is active (its name is printed).
	bool Describe(wipems_openems::OperatorView& view) const;

protected:
	Operator_CUDA();
};

#endif // OPERATOR_CUDA_H

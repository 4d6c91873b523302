// Replacement for the reference's SparqlResult.cu in the reference-as-oracle
// build (test infrastructure only).  SparqlResult::setResult (declared at
// src/SparqlResult.h:13) is called by QueryPlan::execute with the final IR,
// which QueryPlan's destructor may free before QueryExecutor::query returns
// (a select job owns its IR, src/SelectQueryJob.cu:68-72).  This version
// copies headers and columns out at setResult time so refdriver.cpp can read the
// result after the query; printing is not needed and is a no-op.
#include "SparqlResult.h"

#include <cassert>

SparqlResult::SparqlResult() { resultIR = nullptr; }

void SparqlResult::setResult(IR* ir) {
  resultIR = dynamic_cast<FullRelationIR*>(ir);
  assert(resultIR != nullptr);
  header.clear();
  results.clear();
  for (size_t c = 0; c < resultIR->getColumnNum(); ++c) {
    header.push_back(resultIR->getHeader(c));
    TYPEID_DEVICE_VEC* col = resultIR->getRelation(c);
    results.emplace_back(col->begin(), col->end());
  }
}

FullRelationIR* SparqlResult::getResultIR() { return resultIR; }
std::vector<std::string> SparqlResult::getHeaderVariables() { return header; }
std::vector<std::vector<TYPEID>> SparqlResult::get() { return results; }
std::vector<TYPEID> SparqlResult::get(size_t i) { return results[i]; }
void SparqlResult::printResult(REVERSE_DICTTYPE&, REVERSE_DICTTYPE&, REVERSE_DICTTYPE&) const {}
